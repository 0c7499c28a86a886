"""The C ABI library: loads, exports every function include/*.h declares, and the
ctypes struct layouts agree with the C compiler's. No GPU calls here."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from pxdock_gb300 import abi, build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*[\w\s\*]+?\b(pxd_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    assert len(declared_functions()) >= 20


def test_library_loads_and_reports_version(lib_path):
    lib = C.CDLL(lib_path)
    lib.pxd_abi_version.restype = C.c_int32
    lib.pxd_version.restype = C.c_char_p
    assert lib.pxd_abi_version() == 2
    assert b"sm_103a" in lib.pxd_version()


def test_decide_grid_dims_matches_reference_rule(lib_path):
    """grid.cpp:65-86: 20 A @ 0.375 -> 55 points, 30 A -> 81, 18 A -> 49."""
    lib = C.CDLL(lib_path)
    lib.pxd_decide_grid_dims.argtypes = [C.c_double] * 7 + [C.POINTER(abi.Box)]
    for size, npts in ((20.0, 55), (30.0, 81), (18.0, 49), (0.9, 5)):
        b = abi.Box()
        assert lib.pxd_decide_grid_dims(1.0, 2.0, 3.0, size, size, size, 0.375, C.byref(b)) == 0
        assert list(b.npoints) == [npts] * 3
        assert abs(b.init_xyz[0] - (1.0 - (npts - 1) * 0.375 / 2)) < 1e-12
    assert lib.pxd_decide_grid_dims(0, 0, 0, 1, 1, 1, 0.0, C.byref(abi.Box())) != 0


def test_struct_layouts_match_c_compiler():
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "pxdock_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(pxd_topology), sizeof(pxd_torsion_tree),
         sizeof(pxd_ligand_desc), sizeof(pxd_receptor_desc), sizeof(pxd_box),
         sizeof(pxd_lbfgs_params));
  printf("%zu %zu %zu\n", offsetof(pxd_topology, pairs), offsetof(pxd_ligand_desc, tree),
         offsetof(pxd_lbfgs_params, reset_threshold));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe], check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = [int(v) for v in lines[0].split()]
    assert sizes == [C.sizeof(abi.Topology), C.sizeof(abi.TorsionTree), C.sizeof(abi.LigandDesc),
                     C.sizeof(abi.ReceptorDesc), C.sizeof(abi.Box), C.sizeof(abi.LbfgsParams)]
    offs = [int(v) for v in lines[1].split()]
    assert offs == [abi.Topology.pairs.offset, abi.LigandDesc.tree.offset,
                    abi.LbfgsParams.reset_threshold.offset]
