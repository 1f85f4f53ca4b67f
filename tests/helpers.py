"""Shared test helpers: golden-fixture systems and error metrics."""
from __future__ import annotations

import json
import os

import numpy as np

from gmxapi_gb300.systems import System

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ulp_distance(a, b) -> np.ndarray:
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def rel_rms(f, ref) -> float:
    f = np.asarray(f, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((f - ref) ** 2)) / np.sqrt(np.mean(ref**2)))


def nblib_golden_system(key: str) -> tuple[System, np.ndarray]:
    """The nblib test system and its golden forces (tests/golden/nblib_golden.json).

    C6/C12 are combined geometrically in single precision like
    nblib's ParticleTypesInteractions (api/nblib/interactions.cpp:83-93).
    """
    d = json.load(open(os.path.join(GOLDEN, "nblib_golden.json")))[key]
    n = len(d["x"])
    c6 = np.array(d["c6"], np.float32)
    c12 = np.array(d["c12"], np.float32)
    C6 = np.sqrt(c6[:, None] * c6[None, :]).astype(np.float32)
    C12 = np.sqrt(c12[:, None] * c12[None, :]).astype(np.float32)
    nbfp = np.stack([np.float32(6) * C6, np.float32(12) * C12], -1).reshape(-1).astype(np.float32)
    mol_of = {}
    for m in d["molecules"]:
        for a in m:
            mol_of[a] = m
    ei, el = [0], []
    for a in range(n):
        el += sorted(mol_of[a])
        ei.append(len(el))
    s = System(
        x=np.array(d["x"], np.float32),
        box=np.full(3, d["box"], np.float32),
        q=np.array(d["q"], np.float32),
        type=np.array(d["types"], np.int32),
        ntypes=len(c6),
        nbfp=nbfp,
        excl_index=np.array(ei, np.int32),
        excl_list=np.array(el, np.int32),
        name=key,
    )
    return s, np.array(d["forces"], np.float32)


def canonical_pairs(sci, cj4, excl):
    """Sorted structured array of (sci, shift, i-cluster, j-cluster, 64-bit mask).

    The GPU list stores, per cj4 and warp half, an 8x4 i-cluster/j-cluster
    bit mask and a 32x32-bit exclusion entry.  This expands it to one row per
    interacting cluster pair with a 64-bit atom-pair mask (bit ic*8+jc), the
    layout-independent content compared between implementations.
    """
    sci = np.asarray(sci, np.int64).reshape(-1, 4)
    cj4 = np.asarray(cj4, np.int64).reshape(-1, 8)
    excl = np.asarray(excl, np.uint32).reshape(-1, 32)
    counts = sci[:, 3] - sci[:, 2]
    owner = np.repeat(np.arange(len(sci)), counts)
    j4idx = np.concatenate([np.arange(a, b) for a, b in sci[:, 2:4]]) if len(sci) else np.zeros(0, np.int64)
    out = []
    chunk = 20000
    bits = np.arange(32, dtype=np.uint32)
    for c0 in range(0, len(j4idx), chunk):
        jj = j4idx[c0:c0 + chunk]
        ow = owner[c0:c0 + chunk]
        e = cj4[jj]
        im = [e[:, 4].astype(np.uint32), e[:, 6].astype(np.uint32)]
        # (n, 32 bits) interaction bit per half
        imb = [((m[:, None] >> bits[None, :]) & 1).astype(bool) for m in im]
        # (n, 32 words, 32 bits) exclusion bits per half
        exb = [((excl[e[:, 5 + 2 * h]][:, :, None] >> bits[None, None, :]) & 1).astype(bool) for h in (0, 1)]
        # mask[n, bit, ic, jc]
        mask = np.zeros((len(jj), 32, 8, 8), dtype=bool)
        for jc in range(8):
            h = jc // 4
            w = (jc & 3) * 8 + np.arange(8)  # word index per ic
            mask[:, :, :, jc] = exb[h][:, w, :].transpose(0, 2, 1) & imb[h][:, :, None]
        anyb = imb[0] | imb[1]
        packed = np.packbits(mask.reshape(len(jj), 32, 64), axis=-1, bitorder="little")
        m64 = packed.view(np.uint64).reshape(len(jj), 32)
        n_idx, b_idx = np.nonzero(anyb)
        jm = b_idx // 8
        i = b_idx % 8
        s_ = sci[ow[n_idx]]
        rec = np.empty(len(n_idx), dtype=[("sci", "i8"), ("shift", "i8"), ("ci", "i8"), ("cj", "i8"), ("mask", "u8")])
        rec["sci"] = s_[:, 0]
        rec["shift"] = s_[:, 1]
        rec["ci"] = s_[:, 0] * 8 + i
        rec["cj"] = e[n_idx, jm]
        rec["mask"] = m64[n_idx, b_idx]
        out.append(rec)
    if not out:
        return np.zeros(0, dtype=[("sci", "i8"), ("shift", "i8"), ("ci", "i8"), ("cj", "i8"), ("mask", "u8")])
    allr = np.concatenate(out)
    return np.sort(allr, order=["sci", "shift", "ci", "cj"])
