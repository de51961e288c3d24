"""The Fortran side of the C ABI (fortran/).

* Every `bind(C, name=...)` in the ISO_C_BINDING module names an entry point
  that include/cody_gpu.h declares and libcodygpu.so exports, and the bind(C)
  descriptor type lists the fields of cgpu_desc in order (CPU).
* Where gfortran exists, the module and a small Fortran host program build
  against the library and run one split step on the GPU.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FDIR = os.path.join(ROOT, "fortran")


def _header_text():
    with open(os.path.join(ROOT, "include", "cody_gpu.h")) as f:
        return f.read()


def test_fortran_bindings_name_declared_and_exported_entry_points():
    from codyfortran_gb300 import build
    lib = ctypes.CDLL(build.build())
    header = _header_text()
    names = set()
    for fn in os.listdir(FDIR):
        if fn.endswith(".f90"):
            names |= set(re.findall(r'bind\(C, name="(cgpu_\w+)"\)', open(os.path.join(FDIR, fn)).read()))
    assert len(names) >= 25
    for n in sorted(names):
        assert re.search(rf"\b{n}\(", header), n
        getattr(lib, n)


def test_fortran_descriptor_matches_cgpu_desc():
    src = open(os.path.join(FDIR, "M_CodyGpu.f90")).read()
    body = src.split("type, bind(C) :: T_CgpuDesc", 1)[1].split("end type", 1)[0]
    fields = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if "::" in line:
            for part in re.split(r",\s*(?![^(]*\))", line.split("::", 1)[1]):
                fields.append(part.split("=")[0].split("(")[0].strip())
    header = _header_text()
    cdesc = header.split("typedef struct {", 2)[2].split("} cgpu_desc;", 1)[0]
    cdesc = re.sub(r"/\*.*?\*/", "", cdesc, flags=re.S)
    cfields = []
    for line in cdesc.splitlines():
        line = line.strip().rstrip(";")
        if not line:
            continue
        decl = line.split(None, 1)[1] if not line.startswith("const double*") else line[len("const double*"):]
        for part in decl.split(","):
            cfields.append(part.strip().lstrip("*").split("[")[0].strip())
    assert fields == cfields


@pytest.mark.gpu
def test_fortran_host_program_runs_a_split_step():
    if shutil.which("gfortran") is None:
        pytest.skip("no gfortran on this machine")
    from codyfortran_gb300 import build
    build.build()
    r = subprocess.run(["make", "-s", "-C", FDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([os.path.join(FDIR, "_build", "abi_check")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "abi_check OK" in r.stdout, r.stdout + r.stderr
