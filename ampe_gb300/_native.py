"""Loader and prototypes of libampe_gb300.so (the C-ABI of include/ampe_gb300.h).

The product path has no fallback: if the shared library is missing or
cannot be loaded, importing this module raises.  Build it with
``python -m ampe_gb300.build`` (or ``__graft_entry__.build()``).
"""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libampe_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        "libampe_gb300.so not built (%s); run python -m ampe_gb300.build" % LIB_PATH
    )

lib = C.CDLL(LIB_PATH)

P = C.c_void_p
D = C.c_double
I = C.c_int
MP = C.POINTER(abi.Model)
SP = C.POINTER(abi.StepParams)
MOB = C.POINTER(abi.Mobility)

_PROTOS = {
    "ampe_version": (C.c_char_p, []),
    "ampe_device_count": (I, []),
    "ampe_fill_ghosts": (I, [MP, P, P]),
    "ampe_phase_flux": (I, [MP, P, P, P, P, P, P]),
    "ampe_computerhspbg": (I, [MP, P, P, P, P, P, P, P, P]),
    "ampe_add_driving_force": (I, [MP, P, P, P, P, P, P]),
    "ampe_phase_concentrations": (I, [MP, P, P, P, P, P, P, P, P, P]),
    "ampe_conc_diffusion": (I, [MP, P, P, P, P, P, P, P, P, P]),
    "ampe_add_flux": (I, [MP, P, P, P, P, P, P, P, P]),
    "ampe_conc_flux_kks": (I, [MP, P, P, P, P, P, P, P, P, P]),
    "ampe_computerhsconcentration": (I, [MP, P, P, P, P, P]),
    "ampe_add_flux_from_grad_t": (I, [MP, P, P, P, P, P, P, P, P]),
    "ampe_kim_mobility": (I, [MP, P, P, P, D, D, D, P, P]),
    "ampe_conc_diffusion_mobility": (I, [MP, MOB] + [P] * 17),
    "ampe_fac2_work_doubles": (C.c_longlong, [C.POINTER(abi.Fac2)]),
    "ampe_fac2_composite_residual": (I, [C.POINTER(abi.Fac2), C.POINTER(abi.Fac2Level),
                                         C.POINTER(abi.Fac2Level)] + [P] * 9),
    "ampe_fac2_solve": (I, [C.POINTER(abi.Fac2), C.POINTER(abi.Fac2Level),
                            C.POINTER(abi.Fac2Level), P, P, P, P, I, D, P, P, P]),
    "ampe_quat_symm_table": (I, [P, P]),
    "ampe_quat_symm_rotation": (I, [MP, P, P, P, P, P]),
    "ampe_quat_fundamental": (I, [MP, P, P]),
    "ampe_quat_diffs_symm": (I, [MP, P, P, P, P, P, P, P, P]),
    "ampe_quat_grad_side_symm": (I, [MP] + [P] * 16),
    "ampe_add_flux_from_antitrapping": (I, [MP, P, P, P, P, D, P, P, P, P]),
    "ampe_rhs_phase_conc": (I, [MP, P, P, P, P, P, P, P, P]),
    "ampe_efo_rbgs": (I, [MP, P, P, P, D, P, D, P, D, P, P, I, P, P]),
    "ampe_efo_residual": (I, [MP, P, P, P, D, P, D, P, D, P, P, P, P]),
    "ampe_efo_rbgs_sweep": (I, [MP, P, P, P, D, P, D, P, D, P, P, P, P]),
    "ampe_phase_fac_set_c": (I, [MP, P, D, P, P]),
    "ampe_quat_grad_modulus": (I, [MP, P, P, P]),
    "ampe_quat_mobility": (I, [MP, P, P, P]),
    "ampe_quat_face_coef": (I, [MP, P, P, P, P, P, P, P]),
    "ampe_quat_rhs": (I, [MP, P, P, P, P, P, P, P]),
    "ampe_efo_residual_rms_scratch_doubles": (C.c_size_t, [MP]),
    "ampe_efo_residual_rms": (I, [MP, P, P, P, D, P, D, P, D, P, P, P, P, P]),
    "ampe_efo_residual_rms_noalloc": (I, [MP, P, P, P, D, P, D, P, D, P, P, P, P]),
    "ampe_stepper_create": (I, [MP, SP, C.POINTER(P)]),
    "ampe_stepper_destroy": (I, [P]),
    "ampe_stepper_set_state": (I, [P, P, P, P, P, P, I]),
    "ampe_stepper_get_state": (I, [P, P, P, P, P, I]),
    "ampe_stepper_advance": (I, [P, I, C.POINTER(abi.StepStats)]),
    "ampe_stepper_advance_to": (I, [P, D, I, C.POINTER(abi.StepStats)]),
    "ampe_stepper_set_temperature": (I, [P, D, D]),
    "ampe_stepper_eval_rhs": (I, [P, P, P, I]),
    "ampe_stepper_kernel_launches": (C.c_longlong, [P]),
    "ampe_stepper_load_y": (I, [P, P, P, I]),
    "ampe_stepper_jv": (I, [P, P, D, P, I]),
    "ampe_stepper_set_quat": (I, [P, P, I]),
    "ampe_stepper_set_orientation": (I, [P, P, I]),
    "ampe_stepper_get_quat": (I, [P, P, I]),
    "ampe_stepper_size": (C.c_longlong, [P]),
    "ampe_stepper_eval_rhs_full": (I, [P, P, I]),
    "ampe_stepper_stream": (P, [P]),
    "ampe_stepper_set_stream": (I, [P, P]),
    "ampe_stepper_profile": (I, [P, I]),
    "ampe_stepper_kernel_time": (I, [P, I, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "ampe_stepper_attach_surrogate": (I, [P, P]),
    "ampe_mlp_create": (I, [MP, I, C.c_uint, C.POINTER(P)]),
    "ampe_mlp_destroy": (I, [P]),
    "ampe_mlp_nparams": (I, [P]),
    "ampe_mlp_generate": (I, [P, C.c_longlong, C.c_uint, D, D, D, D, C.POINTER(C.c_longlong)]),
    "ampe_mlp_train": (I, [P, I, I, C.c_float, C.POINTER(C.c_float)]),
    "ampe_mlp_grad": (I, [P, P, P, I, C.POINTER(C.c_float)]),
    "ampe_mlp_get": (I, [P, P, P, I]),
    "ampe_mlp_set": (I, [P, P, I]),
    "ampe_mlp_set_normalization": (I, [P, D, D]),
    "ampe_mlp_infer": (I, [P, MP, P, P, P, P, P, I, P]),
    "ampe_mlp_status": (I, [P]),
    "ampe_mlp_clear_status": (I, [P]),
    "ampe_mlp_set_wait_limit": (I, [P, I, I]),
}

for _name, (_res, _args) in _PROTOS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED = tuple(_PROTOS)


class AmpeError(RuntimeError):
    pass


def check(rc, what="ampe call"):
    """Raise on a negative status; return the (non-negative) status."""
    if rc < 0:
        names = {
            abi.AMPE_ERR_INVALID: "invalid argument",
            abi.AMPE_ERR_CUDA: "CUDA error",
            abi.AMPE_ERR_NOT_CONVERGED: "not converged",
            abi.AMPE_ERR_NO_DEVICE: "no CUDA device",
        }
        raise AmpeError("%s failed: %s (%d)" % (what, names.get(rc, "?"), rc))
    return rc
