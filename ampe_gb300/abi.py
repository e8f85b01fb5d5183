"""ctypes mirror of the plain-C structs in include/ampe_gb300.h.

The field order and types must match the header exactly; the test suite
checks ``ctypes.sizeof`` against the library's own ``sizeof`` report.
"""
import ctypes as C

AMPE_OK = 0
AMPE_ERR_INVALID = -1
AMPE_ERR_CUDA = -2
AMPE_ERR_NOT_CONVERGED = -3
AMPE_ERR_NO_DEVICE = -4
AMPE_ERR_TOO_LARGE = -5
NOALLOC_SCRATCH_DOUBLES = 1 << 19

FLUX_SIMPLE, FLUX_ISOTROPIC, FLUX_ANISOTROPIC = 0, 1, 2
THERMO_DILUTE, THERMO_CALPHAD = 0, 1
TEMP_CONSTANT, TEMP_GRADIENT, TEMP_FIELD = 0, 1, 2
CONC_EBS, CONC_KKS = 0, 1
DIFF_ARRHENIUS, DIFF_MOBILITY = 0, 1
MAX_TSEG = 6


class GTerm(C.Structure):
    """ampe_gterm_t: piecewise pure-species Gibbs energy G(T)."""

    _fields_ = [("nseg", C.c_int), ("tc", C.c_double * (MAX_TSEG + 1))] + [
        (k, C.c_double * MAX_TSEG)
        for k in ("a", "b", "c", "d2", "d3", "d4", "d7", "dm1", "dm9")
    ]


class Mobility(C.Structure):
    """ampe_mobility_t: CALPHAD atomic mobilities of a binary alloy,
    q[species][phase][qA|qB] = (a0, a1, a2, a3) and
    qq[species][phase][n] = (a0, a1) of q<n>AB (phase 0 liquid, 1 solid)."""

    _fields_ = [("q", C.c_double * 4 * 2 * 2 * 2), ("qq", C.c_double * 2 * 4 * 2 * 2)]


class Model(C.Structure):
    """ampe_model_t."""

    _fields_ = [
        ("dim", C.c_int),
        ("n", C.c_int * 3),
        ("ng", C.c_int),
        ("dx", C.c_double * 3),
        ("flux_type", C.c_int),
        ("epsilon_phi", C.c_double),
        ("aniso_eps", C.c_double),
        ("aniso_k", C.c_int),
        ("qlen", C.c_int),
        ("phase_well_scale", C.c_double),
        ("phase_mobility", C.c_double),
        ("well_type", C.c_char),
        ("energy_interp", C.c_char),
        ("conc_interp", C.c_char),
        ("diff_interp", C.c_char),
        ("avg_type", C.c_char),
        ("orient_interp1", C.c_char),
        ("orient_interp2", C.c_char),
        ("pad0", C.c_char),
        ("with_orient", C.c_int),
        ("misorientation_factor", C.c_double),
        ("epsilon_q", C.c_double),
        ("conc_mobility", C.c_double),
        ("D_liquid", C.c_double),
        ("Q_liquid", C.c_double),
        ("D_solid", C.c_double),
        ("Q_solid", C.c_double),
        ("thermo", C.c_int),
        ("inv_molar_volume", C.c_double * 2),
        ("dilute_Tm", C.c_double),
        ("dilute_m", C.c_double),
        ("dilute_k", C.c_double),
        ("g", (GTerm * 2) * 2),
        ("L", ((C.c_double * 2) * 4) * 2),
        ("newton_max_its", C.c_int),
        ("newton_tol", C.c_double),
        ("temp_mode", C.c_int),
        ("T0", C.c_double),
        ("gradT", C.c_double),
        ("evolve_quat", C.c_int),
        ("quat_mobility", C.c_double),
        ("min_quat_mobility", C.c_double),
        ("quat_grad_floor", C.c_double),
        ("quat_floor_type", C.c_char),
        ("quat_mobility_type", C.c_char),
        ("pad1", C.c_char * 6),
        ("conc_form", C.c_int),
        ("ng_side", C.c_int),
        ("conc_diffusion", C.c_int),
        ("pad2", C.c_int),
        ("mobility", Mobility),
        ("dTdt", C.c_double),
        ("T_target", C.c_double),
    ]

    def cells(self):
        return self.n[0] * self.n[1] * (self.n[2] if self.dim == 3 else 1)

    def ghost_shape(self):
        """numpy shape (z, y, x) of a ghosted cell field."""
        g = self.ng
        gz = g if self.dim == 3 else 0
        nz = self.n[2] if self.dim == 3 else 1
        return (nz + 2 * gz, self.n[1] + 2 * g, self.n[0] + 2 * g)

    def interior_shape(self):
        nz = self.n[2] if self.dim == 3 else 1
        return (nz, self.n[1], self.n[0])

    def face_shapes(self):
        """(z, y, x) shapes of the three side arrays, ghost width ng_side
        (no z ghosts in 2D)."""
        g = self.ng_side
        gz = g if self.dim == 3 else 0
        nz = self.n[2] if self.dim == 3 else 1
        nx, ny = self.n[0], self.n[1]
        s = [(nz + 2 * gz, ny + 2 * g, nx + 1 + 2 * g), (nz + 2 * gz, ny + 1 + 2 * g, nx + 2 * g)]
        s.append((nz + 1 + 2 * gz, ny + 2 * g, nx + 2 * g) if self.dim == 3 else (1, 1, 1))
        return s


class Fac2(C.Structure):
    """ampe_fac2_t: a periodic coarse level and one fine box refined by 2."""

    _fields_ = [("coarse", Model), ("lo", C.c_int * 3), ("nbox", C.c_int * 3),
                ("ng_fine", C.c_int), ("level_dx", C.c_int), ("presweeps", C.c_int),
                ("postsweeps", C.c_int), ("coarse_sweeps", C.c_int),
                ("d_const", C.c_double), ("c_const", C.c_double), ("m_const", C.c_double)]

    def fine_model(self):
        """The fine level as a Model: n = 2 nbox, dx / 2, ng = ng_fine."""
        f = Model.from_buffer_copy(self.coarse)
        for d in range(3):
            f.n[d] = 2 * self.nbox[d]
            f.dx[d] = 0.5 * self.coarse.dx[d]
        f.ng = self.ng_fine
        f.ng_side = 0
        return f


class Fac2Level(C.Structure):
    """ampe_fac2_level_t: face D (3), cell C and M of one level (NULL:
    the constants of ampe_fac2_t)."""

    _fields_ = [("D", C.c_void_p * 3), ("C", C.c_void_p), ("M", C.c_void_p)]


class StepParams(C.Structure):
    """ampe_step_params_t."""

    _fields_ = [
        ("dt", C.c_double),
        ("max_order", C.c_int),
        ("atol", C.c_double),
        ("rtol", C.c_double),
        ("max_newton", C.c_int),
        ("newton_coef", C.c_double),
        ("max_krylov", C.c_int),
        ("lin_coef", C.c_double),
        ("precond", C.c_int),
        ("fac_max_cycles", C.c_int),
        ("rb_sweeps", C.c_int),
        ("rb_tol", C.c_double),
        ("mg_levels", C.c_int),
        ("mg_pre", C.c_int),
        ("mg_post", C.c_int),
        ("mg_coarse_sweeps", C.c_int),
        ("precision", C.c_int),
        ("surrogate", C.c_int),
        ("max_retries", C.c_int),
        ("adaptive", C.c_int),
        ("h_max", C.c_double),
        ("h_min", C.c_double),
    ]


class StepStats(C.Structure):
    """ampe_step_stats_t."""

    _fields_ = [
        (k, C.c_longlong)
        for k in (
            "steps",
            "newton_iters",
            "gmres_iters",
            "rhs_evals",
            "precond_solves",
            "precond_setups",
            "fac_cycles",
            "newton_fail",
            "kks_iters",
            "kks_fallback",
            "kks_fail",
            "step_retries",
            "kks_fp64_cells",
        )
    ] + [("t", C.c_double), ("err_test_fails", C.c_longlong), ("h_last", C.c_double),
         ("h_next", C.c_double), ("q_last", C.c_int), ("q_next", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}
