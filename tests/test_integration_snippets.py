"""The C++ units of INTEGRATION.md compile against the public header and
link with the library (no GPU needed: nothing runs).

Every block fenced as c++ in INTEGRATION.md is a complete translation unit
(the hooks a ForestClaw maintainer adds: section 2's single_step_update
replacement, section 3's buffered GPU hook). Each is compiled by g++ with
include/geoflood_gb300.h and tests/integration/forestclaw_stub.h (stand-ins
for the ForestClaw declarations the units use), and the objects are linked
into one shared object against libgeoflood_gb300.so with no undefined
symbol allowed, so a drift between the documented bindings and the header
fails here.
"""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
STUB = ROOT / "tests" / "integration"


def units():
    text = (ROOT / "INTEGRATION.md").read_text()
    return re.findall(r"^```c\+\+\n(.*?)^```", text, flags=re.S | re.M)


def test_integration_has_complete_units():
    us = units()
    assert len(us) >= 2
    assert any("gf_patch_update(" in u for u in us)
    assert any("gf_step_buffer_update(" in u for u in us)


def test_units_compile_and_link(tmp_path, gpu_lib):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    objs = []
    for k, u in enumerate(units()):
        src = tmp_path / f"unit{k}.cpp"
        src.write_text(u)
        obj = tmp_path / f"unit{k}.o"
        r = subprocess.run([gxx, "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                            "-Werror", "-include", str(STUB / "forestclaw_stub.h"),
                            f"-I{ROOT / 'include'}", "-c", str(src), "-o", str(obj)],
                           capture_output=True, text=True)
        assert r.returncode == 0, f"unit {k} does not compile:\n{r.stderr}\n{u}"
        objs.append(str(obj))
    stub = tmp_path / "stub.o"
    subprocess.run([gxx, "-std=c++17", "-fPIC", "-c", str(STUB / "forestclaw_stub.cpp"),
                    f"-I{STUB}", "-o", str(stub)], check=True)
    lib = ROOT / "geoflood_gb300" / "libgeoflood_gb300.so"
    r = subprocess.run([gxx, "-shared", "-o", str(tmp_path / "hooks.so"), *objs, str(stub),
                        f"-L{lib.parent}", "-lgeoflood_gb300", "-Wl,--no-undefined",
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, f"link failed:\n{r.stderr}"
