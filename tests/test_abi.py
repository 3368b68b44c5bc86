"""The C ABI library loads and exports every symbol that include/kmhodlr.h declares."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "kmhodlr.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(km_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ("km_partition", "km_create", "km_assemble", "km_factorize", "km_solve", "km_logdet",
              "km_matvec", "km_factor_solve", "km_factor_mul", "km_nll_grad", "km_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from kmhodlr import _lib
    assert set(header_symbols()) == set(_lib.SIGNATURES)


def test_integration_documents_every_entry_point():
    """Every declared entry point has its Julia binding in the shim or in INTEGRATION.md."""
    docs = (ROOT / "INTEGRATION.md").read_text() + (ROOT / "kernelmatrices.jl_gb300" / "julia" / "KMHodlrGPU.jl").read_text()
    missing = [s for s in header_symbols() if s not in docs]
    assert not missing, missing


def test_create_reports_status(lib):
    """km_create either succeeds (a GPU is present) or fails with KM_ERR_CUDA and no handle."""
    import ctypes as C
    from kmhodlr import _lib
    h = C.c_void_p()
    cfg = _lib.KmConfig(device=0, precision=0, hbm_budget_fraction=0.8, refine_max_iter=0, refine_tol=0.0)
    rc = lib.km_create(C.byref(cfg), C.byref(h))
    if rc == _lib.KM_OK:
        assert h.value
        assert lib.km_destroy(h) == _lib.KM_OK
    else:
        assert rc == _lib.KM_ERR_CUDA and not h.value
