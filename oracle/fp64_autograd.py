"""FP64 all-pairs energy functional in torch, differentiated by autograd.

Test infrastructure only: the checker for the adjoint (backward) kernel.  It
is never on the product path.

The energy is the one the cluster-pair kernel integrates, written per pair in
double precision over every atom pair (minimum image; the box must be at least
twice the cut-off):

* LJ with potential shift (reference kernel
  src/gromacs/nbnxm/kernels_reference/kernel_ref_inner.h:141-181):
  E = c12 (r^-12 - rc^-12) / 12 - c6 (r^-6 - rc^-6) / 6 with {c6, c12} =
  {6 C6, 12 C12} from the type table;
* Ewald real space (kernel_ref_inner.h:233-262): E = f q_i q_j (erfc(b r)/r - sh),
  sh = erfc(b rc)/rc with the Ewald potential shift, else 0; excluded pairs
  within the cut-off give -f q_i q_j erf(b r)/r and every atom the self term
  -f b/sqrt(pi) q_i^2 (kernel_gpu_ref.cpp:154-178);
* reaction field (kernel_ref_inner.h:206-231): E = f q_i q_j (1/r + k_rf r^2 - c_rf),
  excluded pairs f q_i q_j (k_rf r^2 - c_rf), self -f c_rf q_i^2 / 2.

Forces are F = -dE/dx by autograd with ``create_graph``, so a scalar loss of
the forces and energies can be differentiated once more with respect to
coordinates, charges and the type table (or per-type sigma/epsilon through a
combination rule).  The pair set is fixed at construction (pairs within the
cut-off at the given coordinates), which is what central differences with a
tiny step need.
"""
from __future__ import annotations

import math

import numpy as np
import torch

COULOMB_EWALD = 0
COULOMB_CUTOFF = 1
COULOMB_RF = 2


def _f32(v):
    return float(np.float32(v))


class AllPairsFP64:
    """The pair set of one system at one configuration, and its energy functional."""

    def __init__(self, system, rc: float, beta: float, epsfac: float, coulomb: int = COULOMB_EWALD,
                 epsilon_rf: float = 1.0, use_ewald_shift: bool = False, x=None):
        x0 = np.asarray(system.x if x is None else x, np.float64)
        box = np.asarray(system.box, np.float64)
        if np.any(box < 2.0 * rc):
            raise ValueError("minimum image needs a box of at least twice the cut-off")
        n = x0.shape[0]
        # the interaction constants are single-precision values in the engine
        rcf = np.float32(rc)
        self.rc = float(rcf)
        self.beta = float(beta)
        self.epsfac = float(epsfac)
        self.coulomb = int(coulomb)
        eps = np.float32(1.0 if coulomb == COULOMB_CUTOFF else epsilon_rf)
        if eps == 0:
            k_rf = np.float32(1) / (np.float32(2) * rcf * rcf * rcf)
        else:
            k_rf = (eps - np.float32(1)) / (np.float32(2) * eps + np.float32(1)) / (rcf * rcf * rcf)
        self.k_rf = float(k_rf)
        self.c_rf = float(np.float32(1) / rcf + k_rf * rcf * rcf)
        self.sh_ewald = math.erfc(self.beta * self.rc) / self.rc if use_ewald_shift else 0.0
        excl = set()
        for i in range(n):
            for k in range(int(system.excl_index[i]), int(system.excl_index[i + 1])):
                j = int(system.excl_list[k])
                if j > i:
                    excl.add((i, j))
        ii, jj, ss, ex = [], [], [], []
        rc2 = self.rc * self.rc
        for i0 in range(0, n, 256):
            i1 = min(n, i0 + 256)
            d = x0[i0:i1, None, :] - x0[None, :, :]
            s = -np.round(d / box)
            d = d + s * box
            r2 = np.einsum("abk,abk->ab", d, d)
            a, b = np.nonzero(r2 < rc2)
            keep = (a + i0) < b
            a, b = a[keep] + i0, b[keep]
            ii.append(a)
            jj.append(b)
            ss.append(s[a - i0, b])
        self.i = torch.from_numpy(np.concatenate(ii).astype(np.int64))
        self.j = torch.from_numpy(np.concatenate(jj).astype(np.int64))
        self.shift = torch.from_numpy(np.concatenate(ss) * box)
        ex = np.array([(int(a), int(b)) in excl for a, b in zip(self.i.tolist(), self.j.tolist())], bool)
        self.excluded = torch.from_numpy(ex)
        self.type = torch.from_numpy(np.asarray(system.type, np.int64))
        self.n = n

    def energies(self, x: torch.Tensor, q: torch.Tensor, nbfp: torch.Tensor):
        """(E_lj, E_coul) for x (N, 3), q (N,), nbfp (nt, nt, 2), all float64."""
        d = x[self.i] - x[self.j] + self.shift
        r2 = (d * d).sum(-1)
        r = torch.sqrt(r2)
        keep = ~self.excluded
        ti, tj = self.type[self.i], self.type[self.j]
        c6 = nbfp[ti, tj, 0]
        c12 = nbfp[ti, tj, 1]
        rinv6 = 1.0 / (r2 * r2 * r2)
        rc6 = self.rc**-6
        e_lj = c12 * (rinv6 * rinv6 - rc6 * rc6) / 12.0 - c6 * (rinv6 - rc6) / 6.0
        e_lj = torch.where(keep, e_lj, torch.zeros_like(e_lj)).sum()
        qq = self.epsfac * q[self.i] * q[self.j]
        if self.coulomb == COULOMB_EWALD:
            br = self.beta * r
            e_pair = torch.where(keep, torch.special.erfc(br) / r - self.sh_ewald, -torch.erf(br) / r)
            e_self = -self.epsfac * self.beta / math.sqrt(math.pi) * (q * q).sum()
        else:
            e_pair = torch.where(keep, 1.0 / r, torch.zeros_like(r)) + self.k_rf * r2 - self.c_rf
            e_self = -0.5 * self.epsfac * self.c_rf * (q * q).sum()
        e_c = (qq * e_pair).sum() + e_self
        return e_lj, e_c

    def forces_energies(self, x: torch.Tensor, q: torch.Tensor, nbfp: torch.Tensor):
        """Forces (N, 3) = -dE/dx (kept differentiable) and [E_lj, E_coul]."""
        if not x.requires_grad:
            x = x.requires_grad_(True)
        e_lj, e_c = self.energies(x, q, nbfp)
        (g,) = torch.autograd.grad(e_lj + e_c, x, create_graph=True)
        return -g, torch.stack((e_lj, e_c))
