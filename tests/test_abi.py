"""The C-ABI library: builds for sm_103a, loads, exports what the header declares (no GPU needed)."""
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "nbnxm_gb300.h")).read()
    decl = r"^(?:const\s+)?(?:int|void|char|float|double)\s*\*?\s*(nbx_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.M)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_builds_and_exports_header_symbols():
    from gmxapi_gb300 import _lib, build

    build.build()
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(_lib.EXPORTED) == syms


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from gmxapi_gb300 import _lib

    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()


def test_create_without_gpu_reports_no_device():
    """Without a GPU the engine refuses with NBX_ERR_NO_DEVICE instead of computing on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gmxapi_gb300 import _lib, nblib, systems

    s = systems.spc_water(30, 1.0, seed=1)
    with pytest.raises(_lib.NbxError) as ei:
        nblib.ForceCalculator(s)
    assert ei.value.code == 6
