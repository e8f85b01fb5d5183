"""C-ABI surface checks that need no GPU: the library loads, exports every
function include/ampe_gb300.h declares, its structs match the ctypes
mirrors, and host-side argument validation rejects bad calls before any
kernel launch."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from ampe_gb300 import abi, configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ampe_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ampe_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from ampe_gb300 import _native

    decl = declared_functions()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(_native.lib, name), name
    assert set(decl) == set(_native.EXPORTED)
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH],
                         capture_output=True, text=True).stdout
    for name in decl:
        assert re.search(r"\bT %s\b" % name, out), name


def test_struct_layout_matches_header():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "ampe_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(ampe_model_t),
         sizeof(ampe_gterm_t), sizeof(ampe_step_params_t),
         sizeof(ampe_step_stats_t), offsetof(ampe_model_t, g),
         offsetof(ampe_model_t, T0), offsetof(ampe_step_params_t, max_retries));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        exe = os.path.join(d, "s")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    assert vals == [
        C.sizeof(abi.Model),
        C.sizeof(abi.GTerm),
        C.sizeof(abi.StepParams),
        C.sizeof(abi.StepStats),
        abi.Model.g.offset,
        abi.Model.T0.offset,
        abi.StepParams.max_retries.offset,
    ]


def test_argument_validation_without_gpu():
    from ampe_gb300 import _native

    L = _native.lib
    m = configs.dilute2d(16)
    bad = configs.dilute2d(16)
    bad.dim = 4
    assert L.ampe_fill_ghosts(C.byref(bad), C.c_void_p(1), None) == abi.AMPE_ERR_INVALID
    assert L.ampe_fill_ghosts(C.byref(m), None, None) == abi.AMPE_ERR_INVALID
    iso3 = configs.calphad3d(8)
    iso3.flux_type = abi.FLUX_ISOTROPIC  # no 3D isotropic stencil in the reference
    assert L.ampe_phase_flux(C.byref(iso3), C.c_void_p(1), None, C.c_void_p(1),
                             C.c_void_p(1), C.c_void_p(1), None) == abi.AMPE_ERR_INVALID
    small = configs.dilute2d(16)
    small.n[0] = 1  # fewer cells than twice the ghost width
    assert L.ampe_efo_rbgs(C.byref(small), None, None, None, 1.0, None, 1.0, None, 1.0,
                           C.c_void_p(1), C.c_void_p(1), 0, None, None) == abi.AMPE_ERR_INVALID
    assert L.ampe_efo_rbgs(C.byref(m), None, None, None, 1.0, None, 1.0, None, 1.0,
                           C.c_void_p(1), C.c_void_p(1), 2, None, None) == abi.AMPE_ERR_INVALID


def test_stepper_create_reports_missing_device_or_bad_params():
    from ampe_gb300 import _native

    L = _native.lib
    m = configs.dilute2d(16)
    p = configs.step_params()
    p.dt = -1.0
    h = C.c_void_p()
    assert L.ampe_stepper_create(C.byref(m), C.byref(p), C.byref(h)) == abi.AMPE_ERR_INVALID
    if L.ampe_device_count() == 0:
        p = configs.step_params()
        assert L.ampe_stepper_create(C.byref(m), C.byref(p), C.byref(h)) == abi.AMPE_ERR_NO_DEVICE


def test_version_string():
    from ampe_gb300 import _native

    assert b"sm_103a" in _native.lib.ampe_version()


@pytest.mark.parametrize("case", ["krylov", "precision", "aniso_evolving_mixed", "aniso_qlen",
                                  "quat_qlen", "quat_mobility", "precond"])
def test_stepper_rejects_unsupported_combinations(case):
    """ampe_stepper_create validates the model and the parameters on the
    host, before it looks for a device."""
    from ampe_gb300 import _native

    L = _native.lib
    m = configs.dilute2d(16)
    p = configs.step_params()
    if case == "krylov":
        p.max_krylov = 17  # the Krylov basis is sized for at most 16
    elif case == "precision":
        p.precision = 2
    elif case == "aniso_evolving_mixed":
        m = configs.polycrystal3d(8)
        m.flux_type, m.qlen = abi.FLUX_ANISOTROPIC, 4
        p.precision = 1  # the mixed path linearises the flux for a static orientation only
    elif case == "aniso_qlen":
        m.flux_type, m.qlen = abi.FLUX_ANISOTROPIC, 3
    elif case == "quat_qlen":
        m = configs.polycrystal3d(8)
        m.flux_type, m.qlen = abi.FLUX_ANISOTROPIC, 2
    elif case == "quat_mobility":
        m = configs.polycrystal3d(8)
        m.quat_grad_floor = 0.0
    elif case == "precond":
        p.precond = 3
    h = C.c_void_p()
    assert L.ampe_stepper_create(C.byref(m), C.byref(p), C.byref(h)) == abi.AMPE_ERR_INVALID
    assert not h.value
