"""ctypes access to the CPU oracle (oracle/_build/liborc_ampe.so).

Test infrastructure: the oracle is the checker of the CUDA library and is
only loaded by tests, __graft_entry__.smoke() and bench.py's CPU baseline.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liborc_ampe.so")

import sys  # noqa: E402

sys.path.insert(0, ROOT)
from ampe_gb300 import abi  # noqa: E402


def build_oracle():
    subprocess.run(["make", "-C", ORACLE_DIR, "-j8", "-s"], check=True)
    return ORACLE_LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(ORACLE_LIB)
        P, D, I = C.c_void_p, C.c_double, C.c_int
        MP = C.POINTER(abi.Model)
        SP = C.POINTER(abi.StepParams)
        protos = {
            "orc_interp_func": (D, [D, C.c_char]),
            "orc_deriv_interp_func": (D, [D, C.c_char]),
            "orc_second_deriv_interp_func": (D, [D, C.c_char]),
            "orc_well_func": (D, [D, C.c_char]),
            "orc_deriv_well_func": (D, [D, C.c_char]),
            "orc_second_deriv_well_func": (D, [D, C.c_char]),
            "orc_average_func": (D, [D, D, C.c_char]),
            "orc_free_energy": (D, [MP, D, D, I]),
            "orc_dfdc": (D, [MP, D, D, I]),
            "orc_d2fdc2": (D, [MP, D, D, I]),
            "orc_kks_cell": (I, [MP, D, D, D, P]),
            "orc_ceq": (I, [MP, D, P]),
            "orc_fill_ghosts": (None, [MP, P]),
            "orc_phase_flux": (None, [MP, P, P, P, P, P]),
            "orc_computerhspbg": (None, [MP, P, P, P, P, P, P, P]),
            "orc_add_driving_force": (None, [MP, P, P, P, P, P]),
            "orc_phase_concentrations": (C.c_long, [MP, P, P, P, P, P, P, P, P]),
            "orc_conc_diffusion": (None, [MP, P, P, P, P, P, P, P, P]),
            "orc_add_flux": (None, [MP, P, P, P, P, P, P, P]),
            "orc_computerhsconcentration": (None, [MP, P, P, P, P]),
            "orc_add_flux_from_grad_t": (None, [MP, P, P, P, P, P, P, P]),
            "orc_kim_mobility": (None, [MP, P, P, P, D, D, D, D, P]),
            "orc_phase_diffusion_mobility": (D, [MP, C.POINTER(abi.Mobility), I, D, D]),
            "orc_conc_diffusion_mobility": (None, [MP, C.POINTER(abi.Mobility)] + [P] * 16),
            "orc_conc_diffusion_model": (None, [MP] + [P] * 10),
            "orc_fac2_work_doubles": (C.c_longlong, [C.POINTER(abi.Fac2)]),
            "orc_fac2_composite_residual": (D, [C.POINTER(abi.Fac2), P, P] + [P] * 6),
            "orc_fac2_solve": (I, [C.POINTER(abi.Fac2), P, P, P, P, P, P, I, D, P]),
            "orc_quat_symm_table": (None, [P, P]),
            "orc_quat_find_symm": (I, [P, P, I, P]),
            "orc_quat_symm_rotation": (None, [MP, P, P, P, P]),
            "orc_quat_fundamental": (None, [MP, P]),
            "orc_quat_diffs_symm": (None, [MP] + [P] * 7),
            "orc_quat_grad_side_symm": (None, [MP] + [P] * 15),
            "orc_add_flux_from_antitrapping": (None, [MP, P, P, P, P, D, P, P, P]),
            "orc_conc_flux_kks": (None, [MP, P, P, P, P, P, P, P, P, P]),
            "orc_rhs_phase_conc": (None, [MP, P, P, P, P, P, P, P, P]),
            "orc_efo_rbgs": (D, [MP, P, P, P, D, P, D, P, D, P, P, I]),
            "orc_efo_residual": (None, [MP, P, P, P, D, P, D, P, D, P, P, P]),
            "orc_phase_fac_set_c": (None, [MP, P, D, P]),
            "orc_rms_interior": (D, [MP, P]),
            "orc_fac_create": (P, [MP, I]),
            "orc_fac_destroy": (None, [P]),
            "orc_fac_set_operator": (None, [P, P, P, P, D, P, D, P, D]),
            "orc_fac_solve": (I, [P, SP, I, P, P, D, P]),
            "orc_stepper_create": (P, [MP, SP]),
            "orc_stepper_destroy": (None, [P]),
            "orc_stepper_set_state": (None, [P, P, P, P, P, P]),
            "orc_stepper_get_state": (None, [P, P, P, P, P]),
            "orc_stepper_eval_rhs": (None, [P, P, P]),
            "orc_stepper_advance": (I, [P, I, C.POINTER(abi.StepStats)]),
            "orc_stepper_advance_to": (I, [P, D, I, C.POINTER(abi.StepStats)]),
            "orc_stepper_set_temperature": (None, [P, D, D]),
            "orc_stepper_jv": (None, [P, P, D, P, I]),
            "orc_stepper_set_quat": (None, [P, P]),
            "orc_stepper_get_quat": (None, [P, P]),
            "orc_quat_grad_modulus": (None, [MP, P, P]),
            "orc_quat_mobility": (None, [MP, P, P]),
            "orc_quat_face_coef": (None, [MP, P, P, P, P, P, P]),
            "orc_quat_rhs": (None, [MP, P, P, P, P, P, P]),
            "orc_stepper_eval_rhs_full": (None, [P, P]),
            "orc_stepper_set_orientation": (None, [P, P]),
            "orc_stepper_size": (C.c_long, [P]),
            "orc_rhs_phase_conc_q": (None, [MP, P, P, P, P, P, P, P, P, P]),
            "orc_jv_analytic": (None, [MP, P, P, P, P, D, P]),
        }
        for name, (res, args) in protos.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class OracleStepper:
    def __init__(self, model, params):
        self.L = lib()
        self.model = model
        self.h = self.L.orc_stepper_create(C.byref(model), C.byref(params))
        self.n = model.cells()

    def close(self):
        if self.h:
            self.L.orc_stepper_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, phi, c, cl=None, cs=None, temp=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64)
             for x in (phi, c, cl, cs, temp)]
        self.L.orc_stepper_set_state(self.h, *[ptr(x) for x in a])

    def set_quat(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        self.L.orc_stepper_set_quat(self.h, ptr(q))

    def set_orientation(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._q_keep = q
        self.L.orc_stepper_set_orientation(self.h, ptr(q))

    def get_quat(self):
        q = np.empty((4,) + tuple(self.model.interior_shape()))
        self.L.orc_stepper_get_quat(self.h, ptr(q))
        return q

    def get_state(self):
        out = [np.empty(self.n) for _ in range(4)]
        self.L.orc_stepper_get_state(self.h, *[ptr(x) for x in out])
        shp = self.model.interior_shape()
        return tuple(x.reshape(shp) for x in out)

    def eval_rhs(self):
        fp, fc = np.empty(self.n), np.empty(self.n)
        self.L.orc_stepper_eval_rhs(self.h, ptr(fp), ptr(fc))
        shp = self.model.interior_shape()
        return fp.reshape(shp), fc.reshape(shp)

    def eval_rhs_full(self):
        out = np.empty(self.L.orc_stepper_size(self.h))
        self.L.orc_stepper_eval_rhs_full(self.h, ptr(out))
        return out

    def jv(self, v, gamma, analytic):
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        out = np.empty_like(v)
        self.L.orc_stepper_jv(self.h, ptr(v), gamma, ptr(out), int(analytic))
        return out

    def advance(self, n):
        st = abi.StepStats()
        rc = self.L.orc_stepper_advance(self.h, int(n), C.byref(st))
        return rc, st.as_dict()

    def advance_to(self, t_stop, max_steps=1):
        st = abi.StepStats()
        rc = self.L.orc_stepper_advance_to(self.h, float(t_stop), int(max_steps), C.byref(st))
        return rc, st.as_dict()

    def set_temperature(self, T0, gradT=0.0):
        self.L.orc_stepper_set_temperature(self.h, float(T0), float(gradT))


def ghosted(model, interior):
    """Interior (z,y,x) array -> ghosted array with periodic ghosts."""
    g = model.ng
    gz = g if model.dim == 3 else 0
    pad = ((gz, gz), (g, g), (g, g))
    return np.ascontiguousarray(np.pad(interior, pad, mode="wrap"))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return num / den if den > 0 else num
