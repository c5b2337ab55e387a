"""The C ABI without a GPU: the library loads, exports every entry point the
headers declare, the Python mirror of the structs and enums matches the C
layout, and the product path fails loudly instead of falling back."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from wrf_gb300 import abi
from wrf_gb300 import gpu as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
HEADERS = ["wrfgpu.h", "wrfgpu_fortran.h"]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(os.path.join(INC, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?(?:int|long long|char\s*\*|const char\s*\*)\s*\*?\s*(wrfgpu_\w+)\s*\(",
                            src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(G.lib_path()):
        import __graft_entry__ as g
        g.build()
    return C.CDLL(G.lib_path())


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 35, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_header():
    """Compile a probe against the header and compare sizes / offsets with the
    ctypes mirror used by the Python front end."""
    probe = r'''
#include <stdio.h>
#include <stddef.h>
#include "wrfgpu.h"
int main(void) {
  printf("%zu %zu %zu\n", sizeof(WrfDynConfig), sizeof(WrfGpuScalars), sizeof(WrfGpuDomainDesc));
  printf("%zu %zu %zu\n", offsetof(WrfGpuDomainDesc, config), offsetof(WrfGpuDomainDesc, scalars),
         offsetof(WrfDynConfig, time_step_sound));
  printf("%d %d %d %d %d\n", WRFGPU_N3D, WRFGPU_N2D, WRFGPU_N1D, WRFGPU_SPECIES_BASE, WRFGPU_R_RK_TENDENCY);
  printf("%d %d %d\n", WRFGPU_MUTS, WRFGPU_RDNW, WRFGPU_ADVECT_TEND);
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(src, "w").write(probe)
        subprocess.run(["gcc", "-I", INC, "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = [int(v) for v in out]
    assert vals[0] == C.sizeof(abi.WrfDynConfig)
    assert vals[1] == C.sizeof(abi.WrfGpuScalars)
    assert vals[2] == C.sizeof(abi.WrfGpuDomainDesc)
    assert vals[3] == abi.WrfGpuDomainDesc.config.offset
    assert vals[4] == abi.WrfGpuDomainDesc.scalars.offset
    assert vals[5] == abi.WrfDynConfig.time_step_sound.offset
    assert vals[6] == len(abi.F3D) and vals[7] == len(abi.F2D) and vals[8] == len(abi.F1D)
    assert vals[9] == abi.SPECIES_BASE
    assert vals[10] == abi.ROUTINES["rk_tendency"]
    assert vals[11] == abi.FIELD_ID["muts"] and vals[12] == abi.FIELD_ID["rdnw"]
    assert vals[13] == abi.FIELD_ID["advect_tend"]


def test_routine_ids_match_oracle():
    src = open(os.path.join(ROOT, "oracle", "oracle_routines.h")).read()
    ids = dict((k.lower(), int(v)) for k, v in re.findall(r"ORACLE_R_(\w+)\s*=\s*(\d+)", src))
    assert ids["rk_step_prep"] == abi.ROUTINES["rk_step_prep"]
    assert ids["advance_w"] == abi.ROUTINES["advance_w"]
    assert ids["rk_tendency"] == abi.ROUTINES["rk_tendency"]
    assert ids["calc_p_rho_phi"] == abi.ROUTINES["calc_p_rho_phi"]


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(G, "_LIB", None)
    monkeypatch.setattr(G, "lib_path", lambda: str(tmp_path / "absent.so"))
    with pytest.raises(G.WrfGpuError):
        G.load()


def test_no_device_is_an_error_not_a_fallback(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wrf_gb300 import cases
    case = cases.small_case()
    with pytest.raises(G.WrfGpuError):
        G.Ensemble([case.desc])
