"""Python front end of the C-ABI implicit stepper.

Mirrors how QuatModel drives QuatIntegrator (QuatModel.cc:2318 ->
QuatIntegrator::Advance, QuatIntegrator.cc:2096): set the state, advance a
number of accepted steps of a fixed size, read the state back.
"""
import ctypes as C

import numpy as np

from . import abi
from ._native import check, lib


def _ptr(a):
    """Raw pointer of a contiguous numpy array or CUDA tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"] or a.dtype != np.float64:
            raise ValueError("need a C-contiguous float64 array")
        return a.ctypes.data
    return a.data_ptr()


class ImplicitStepper:
    """One uniform periodic level, phi + c (+ quaternion q when the model
    has evolve_quat), on the current CUDA device."""

    def __init__(self, model, params):
        self.model = model
        self.params = params
        h = C.c_void_p()
        check(lib.ampe_stepper_create(C.byref(model), C.byref(params), C.byref(h)),
              "ampe_stepper_create")
        self._h = h
        self.n = model.cells()

    def close(self):
        if self._h:
            lib.ampe_stepper_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, phi, conc, cl=None, cs=None, temp=None):
        host = isinstance(phi, np.ndarray)
        arrs = [phi, conc, cl, cs, temp]
        if host:
            arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                    for a in arrs]
        self._keep = arrs
        check(lib.ampe_stepper_set_state(self._h, *[_ptr(a) for a in arrs],
                                         1 if host else 0),
              "ampe_stepper_set_state")

    def get_state(self):
        phi = np.empty(self.n)
        c = np.empty(self.n)
        cl = np.empty(self.n)
        cs = np.empty(self.n)
        check(lib.ampe_stepper_get_state(self._h, _ptr(phi), _ptr(c), _ptr(cl),
                                         _ptr(cs), 1), "ampe_stepper_get_state")
        shp = self.model.interior_shape()
        return phi.reshape(shp), c.reshape(shp), cl.reshape(shp), cs.reshape(shp)

    def get_state_device(self, phi, conc):
        check(lib.ampe_stepper_get_state(self._h, _ptr(phi), _ptr(conc), None,
                                         None, 0), "ampe_stepper_get_state")

    def size(self):
        """Length of the state vector y (2N, or 6N with quaternions)."""
        return lib.ampe_stepper_size(self._h)

    def set_quat(self, q):
        """Orientation part of y_n: array (4, *interior shape) of unit
        quaternions, component-major."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.size != 4 * self.n:
            raise ValueError("need 4 x cells values")
        self._keep_q = q
        check(lib.ampe_stepper_set_quat(self._h, _ptr(q), 1), "ampe_stepper_set_quat")

    def set_orientation(self, q):
        """Static orientation of the anisotropic flux: array (qlen, *interior
        shape), component-major."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._keep_o = q
        check(lib.ampe_stepper_set_orientation(self._h, _ptr(q), 1),
              "ampe_stepper_set_orientation")

    def get_quat(self):
        q = np.empty(4 * self.n)
        check(lib.ampe_stepper_get_quat(self._h, _ptr(q), 1), "ampe_stepper_get_quat")
        return q.reshape((4,) + tuple(self.model.interior_shape()))

    def eval_rhs_full(self):
        """f(y_n) for the whole state vector."""
        out = np.empty(self.size())
        check(lib.ampe_stepper_eval_rhs_full(self._h, _ptr(out), 1),
              "ampe_stepper_eval_rhs_full")
        return out

    def eval_rhs(self):
        fp = np.empty(self.n)
        fc = np.empty(self.n)
        check(lib.ampe_stepper_eval_rhs(self._h, _ptr(fp), _ptr(fc), 1),
              "ampe_stepper_eval_rhs")
        shp = self.model.interior_shape()
        return fp.reshape(shp), fc.reshape(shp)

    def jv(self, v, gamma):
        """v - gamma J v at the current state (v: [phi | conc (| q)] interior)."""
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        out = np.empty_like(v)
        check(lib.ampe_stepper_jv(self._h, _ptr(v), float(gamma), _ptr(out), 1),
              "ampe_stepper_jv")
        return out

    def advance(self, nsteps):
        st = abi.StepStats()
        check(lib.ampe_stepper_advance(self._h, int(nsteps), C.byref(st)),
              "ampe_stepper_advance")
        return st.as_dict()

    def advance_to(self, t_stop, max_steps=1):
        """Variable steps (params.adaptive = 1) until t_stop or max_steps
        accepted steps (max_steps = 1: CVODE's one-step mode with a stop
        time)."""
        st = abi.StepStats()
        check(lib.ampe_stepper_advance_to(self._h, float(t_stop), int(max_steps), C.byref(st)),
              "ampe_stepper_advance_to")
        return st.as_dict()

    def set_temperature(self, T0, gradT=0.0):
        check(lib.ampe_stepper_set_temperature(self._h, float(T0), float(gradT)),
              "ampe_stepper_set_temperature")

    def kernel_launches(self):
        return lib.ampe_stepper_kernel_launches(self._h)
