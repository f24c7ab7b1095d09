"""C-ABI checks that need no GPU: the library loads and exports every entry
point declared in include/*.h, and the host-side argument handling behaves."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(gf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "gf_level_step" in names and "gf_patch_update" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [n for n in declared_symbols() if not hasattr(gpu_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header(gpu_lib):
    from geoflood_gb300 import _lib

    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_phys_default_matches_reference_defaults(gpu_lib):
    from geoflood_gb300 import _lib

    p = _lib.gf_phys()
    gpu_lib.gf_phys_default(C.byref(p))
    assert p.grav == 9.81 and p.dry_tolerance == 1e-3
    assert list(p.mthlim) == [4, 4, 4] and p.order == 2 and p.transverse == 2
    assert p.maxcfl_cap == 100.0 and p.num_manning == 1


def test_struct_layout_matches_c():
    from geoflood_gb300 import _lib

    # 4 doubles + 2x4 doubles + 6 ints + 3 ints + 1 int + 1 double
    assert C.sizeof(_lib.gf_phys) == 4 * 8 + 8 * 8 + 10 * 4 + 8


def test_ctx_create_without_gpu_fails_cleanly(gpu_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = gpu_lib.gf_ctx_create(0, C.byref(h))
    assert rc != 0 and not h.value


def test_missing_library_raises(monkeypatch, tmp_path):
    from geoflood_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", tmp_path / "nope.so")
    with pytest.raises(RuntimeError, match="not built"):
        _lib.load()
