"""GB300-native convection-diffusion hot path of ParMooN2022.

Python face of ``libparmoon_cd.so`` (C-ABI in ``include/parmoon_cd.h``): the
host setup hierarchy (TDomain / TFESpace / TStructure of refined unit
squares and cubes), and the CD problem (``ConvectionDiffusion<d>``
assemble / solve / errors) running on the GPU.  Every compute call goes to
the CUDA library; there is no CPU fallback: without the built library or a
CUDA device the calls raise.

Parameter names follow the reference's ParameterDatabase keys
(src/Solver/Solver.C:26-209, src/Multigrid/Multigrid.C:417-509,
src/AssembleRoutines/LocalAssembling.C:564-581).
"""
import ctypes
import os
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libparmoon_cd.so")

CDG_OK = 0
ERRORS = {
    -1: "CDG_ERR_ARG", -2: "CDG_ERR_CUDA", -3: "CDG_ERR_OOM", -4: "CDG_ERR_DIVERGED",
    -5: "CDG_ERR_BREAKDOWN", -6: "CDG_ERR_ZERO_DIAG", -7: "CDG_ERR_PATTERN",
    -8: "CDG_ERR_SINGULAR", -9: "CDG_ERR_NO_DEVICE", -10: "CDG_ERR_LIMIT",
    -11: "CDG_ERR_TIMEOUT",
}
(EX_SINE_LAPLACE, EX_SINE, EX_POLYEXP, EX_CONST_F, EX_POLY1, EX_BUMP, EX_POLY1_T, EX_EXP_SIN,
 EX_LINEAR_ST, EX_QUAD_ST) = range(10)
# TimeDiscretization schemes (db["time_discretization"])
TIME_SCHEMES = {"crank_nicolson": 0, "backward_euler": 1, "bdf_two": 2}
CELL_QUAD, CELL_HEXA, CELL_TETRA = 2, 3, 4

# every symbol include/parmoon_cd.h declares
EXPORTED = [
    "cdg_last_error", "cdg_version", "cdg_context_create", "cdg_context_destroy",
    "cdg_context_synchronize", "cdg_context_launch_count", "cdg_hierarchy_create",
    "cdg_hierarchy_destroy", "cdg_hierarchy_level_info", "cdg_hierarchy_get_mesh",
    "cdg_hierarchy_get_dofs", "cdg_hierarchy_get_pattern", "cdg_problem_create",
    "cdg_problem_create_from_arrays", "cdg_problem_destroy", "cdg_problem_assemble",
    "cdg_problem_solve", "cdg_problem_assemble_solve", "cdg_problem_errors",
    "cdg_problem_level_info", "cdg_problem_operator_layout", "cdg_problem_lattice",
    "cdg_problem_get_matrix", "cdg_problem_get_rhs",
    "cdg_problem_get_solution", "cdg_problem_set_solution", "cdg_problem_get_slots",
    "cdg_problem_apply", "cdg_problem_prolongate", "cdg_problem_restrict",
    "cdg_problem_precondition", "cdg_context_stream", "cdg_problem_time_kernel",
    "cdg_problem_errors_noalloc", "cdg_hierarchy_create_tetra", "cdg_problem_tcd_initialize",
    "cdg_hierarchy_create_device", "cdg_hierarchy_create_tetra_device",
    "cdg_space_number_device", "cdg_structure_build_device",
    "cdg_vector_write_file", "cdg_vector_read_file", "cdg_checkpoint_file_name",
    "cdg_problem_write_solution", "cdg_problem_read_solution", "cdg_problem_checkpoint",
    "cdg_problem_tcd_step", "cdg_problem_get_tcd_matrix", "cdg_server_create",
    "cdg_server_destroy", "cdg_request_ndof", "cdg_server_submit", "cdg_server_wait",
    "cdg_server_counters", "cdg_problem_apply32", "cdg_problem_tuning",
    "cdg_problem_quadrature_points", "cdg_problem_assemble_coefficients",
    "cdg_problem_set_fp32_tensor_levels", "cdg_problem_get_matrix32", "cdg_solve_batched",
    "cdg_server_batch_counters", "cdg_hierarchy_perturb",
]


class CdgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "CDG_ERR"), code, msg))
        self.code = code


class AssemblyParams(ctypes.Structure):
    _fields_ = [
        ("example", ctypes.c_int), ("eps", ctypes.c_double), ("b", ctypes.c_double * 3),
        ("c", ctypes.c_double), ("freq", ctypes.c_double), ("supg", ctypes.c_int),
        ("sdfem_type", ctypes.c_int), ("delta0", ctypes.c_double), ("delta1", ctypes.c_double),
        ("cell_measure", ctypes.c_int), ("problem_linear", ctypes.c_int),
        ("neumann_mask", ctypes.c_int), ("poly_degree", ctypes.c_int),
        ("b_grad", ctypes.c_double * 9), ("t", ctypes.c_double), ("ic", ctypes.c_double * 4),
        ("time_step", ctypes.c_double), ("time_discretization", ctypes.c_int),
        ("bdf_two_first_step", ctypes.c_int),
    ]


class SolverParams(ctypes.Structure):
    _fields_ = [
        ("preconditioner", ctypes.c_int), ("max_n_iterations", ctypes.c_int),
        ("min_n_iterations", ctypes.c_int), ("gmres_restart", ctypes.c_int),
        ("residual_tolerance", ctypes.c_double), ("residual_reduction", ctypes.c_double),
        ("divergence_factor", ctypes.c_double), ("multigrid_n_levels", ctypes.c_int),
        ("multigrid_cycle_type", ctypes.c_int), ("multigrid_n_pre_smooth", ctypes.c_int),
        ("multigrid_n_post_smooth", ctypes.c_int), ("jacobi_damp", ctypes.c_double),
        ("multigrid_correction_damp_factor", ctypes.c_double),
        ("multigrid_smoother_coarse", ctypes.c_int), ("multigrid_coarse_residual", ctypes.c_double),
        ("multigrid_coarse_max_n_iterations", ctypes.c_int), ("precision", ctypes.c_int),
        ("gram_schmidt", ctypes.c_int),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double),
                ("initial_residual", ctypes.c_double), ("seconds", ctypes.c_double)]


class Request(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("order", ctypes.c_int), ("n", ctypes.c_int),
                ("a", AssemblyParams), ("s", SolverParams)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("stats", SolveStats),
                ("queue_seconds", ctypes.c_double), ("latency_seconds", ctypes.c_double),
                ("slot", ctypes.c_int), ("ndof", ctypes.c_int)]


_lib = None


def lib():
    """Load libparmoon_cd.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libparmoon_cd.so is not built (run parmoon2022_gb300/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        P, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        PP = ctypes.POINTER(ctypes.c_void_p)
        L.cdg_last_error.restype = ctypes.c_char_p
        L.cdg_context_launch_count.restype = ctypes.c_longlong
        L.cdg_context_launch_count.argtypes = [P]
        sig = {
            "cdg_version": [], "cdg_context_create": [ctypes.c_int, PP],
            "cdg_context_destroy": [P], "cdg_context_synchronize": [P],
            "cdg_hierarchy_create": [ctypes.c_int] * 6 + [PP], "cdg_hierarchy_destroy": [P],
            "cdg_hierarchy_level_info": [P, ctypes.c_int, ip],
            "cdg_hierarchy_get_mesh": [P, ctypes.c_int, dp],
            "cdg_hierarchy_get_dofs": [P, ctypes.c_int, ip],
            "cdg_hierarchy_get_pattern": [P, ctypes.c_int, ip, ip],
            "cdg_problem_create": [P, P, PP],
            "cdg_problem_create_from_arrays": [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip,
                                               PP, PP, ip, ip, PP, PP, PP, PP],
            "cdg_problem_destroy": [P],
            "cdg_problem_assemble": [P, ctypes.POINTER(AssemblyParams)],
            "cdg_problem_solve": [P, ctypes.POINTER(SolverParams), ctypes.POINTER(SolveStats)],
            "cdg_problem_assemble_solve": [P, ctypes.POINTER(AssemblyParams),
                                           ctypes.POINTER(SolverParams), dp, dp, dp,
                                           ctypes.POINTER(SolveStats)],
            "cdg_problem_errors": [P, ctypes.POINTER(AssemblyParams), dp],
            "cdg_problem_errors_noalloc": [P, ctypes.POINTER(AssemblyParams), dp],
            "cdg_hierarchy_create_tetra": [ctypes.c_int] * 5 + [ctypes.c_double,
                                                                ctypes.c_ulonglong, PP],
            "cdg_hierarchy_create_device": [P] + [ctypes.c_int] * 6 + [PP],
            "cdg_hierarchy_create_tetra_device": [P] + [ctypes.c_int] * 5 + [
                ctypes.c_double, ctypes.c_ulonglong, PP],
            "cdg_space_number_device": [P] + [ctypes.c_int] * 4 + [dp, ip, ip, ip],
            "cdg_vector_write_file": [ctypes.c_char_p, dp, ctypes.c_longlong],
            "cdg_vector_read_file": [ctypes.c_char_p, dp, ctypes.c_longlong, ctypes.c_longlong,
                                     ctypes.POINTER(ctypes.c_longlong)],
            "cdg_checkpoint_file_name": [ctypes.c_char_p, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_char_p, ctypes.c_longlong],
            "cdg_problem_write_solution": [P, ctypes.c_char_p],
            "cdg_problem_read_solution": [P, ctypes.c_char_p],
            "cdg_problem_checkpoint": [P, ctypes.c_char_p, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ip],
            "cdg_structure_build_device": [P] + [ctypes.c_int] * 3 + [
                ip, ip, ip, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)],
            "cdg_problem_tcd_initialize": [P, ctypes.POINTER(AssemblyParams)],
            "cdg_problem_tcd_step": [P, ctypes.POINTER(AssemblyParams), ctypes.c_double,
                                     ctypes.POINTER(SolverParams), ctypes.POINTER(SolveStats)],
            "cdg_problem_get_tcd_matrix": [P, ctypes.c_int, ctypes.c_int, dp],
            "cdg_problem_level_info": [P, ctypes.c_int, ip],
            "cdg_problem_operator_layout": [P, ctypes.c_int, ip,
                                            ctypes.POINTER(ctypes.c_longlong), ip],
            "cdg_problem_lattice": [P, ctypes.c_int, ip, ip],
            "cdg_problem_get_matrix": [P, ctypes.c_int, dp],
            "cdg_problem_get_rhs": [P, ctypes.c_int, dp],
            "cdg_problem_get_solution": [P, dp], "cdg_problem_set_solution": [P, dp],
            "cdg_problem_get_slots": [P, ctypes.c_int, ip],
            "cdg_problem_apply": [P, ctypes.c_int, dp, dp],
            "cdg_problem_tuning": [P, ctypes.c_int, ip, ip, dp],
            "cdg_problem_set_fp32_tensor_levels": [P, ctypes.c_int],
            "cdg_problem_get_matrix32": [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)],
            "cdg_problem_quadrature_points": [P, ctypes.POINTER(AssemblyParams), ctypes.c_int,
                                              ip, dp],
            "cdg_problem_assemble_coefficients": [P, ctypes.POINTER(AssemblyParams),
                                                  ctypes.c_int, dp],
            "cdg_problem_apply32": [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                    ctypes.POINTER(ctypes.c_float)],
            "cdg_problem_prolongate": [P, ctypes.c_int, dp, dp],
            "cdg_problem_restrict": [P, ctypes.c_int, dp, dp],
            "cdg_problem_precondition": [P, ctypes.POINTER(SolverParams), dp, dp],
            "cdg_context_stream": [P, PP],
            "cdg_problem_time_kernel": [P, ctypes.POINTER(AssemblyParams), ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, dp],
            "cdg_server_create": [ctypes.c_int, ctypes.c_int, ctypes.c_longlong, PP],
            "cdg_server_destroy": [P],
            "cdg_request_ndof": [ctypes.POINTER(Request), ip],
            "cdg_server_submit": [P, ctypes.POINTER(Request), dp, ctypes.POINTER(ctypes.c_longlong)],
            "cdg_server_wait": [P, ctypes.c_longlong, ctypes.c_double, ctypes.POINTER(Result)],
            "cdg_server_counters": [P, ctypes.POINTER(ctypes.c_longlong)],
            "cdg_solve_batched": [P, ctypes.c_int, PP, ctypes.POINTER(SolverParams), ip,
                                  ctypes.POINTER(SolveStats)],
            "cdg_server_batch_counters": [P, ctypes.POINTER(ctypes.c_longlong)],
            "cdg_hierarchy_perturb": [P, ctypes.c_double, ctypes.c_ulonglong],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = args
        _lib = L
    return _lib


def _chk(rc):
    if rc != CDG_OK:
        raise CdgError(rc, lib().cdg_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def assembly_params(example=EX_SINE, eps=1.0, b=(0.0, 0.0, 0.0), c=0.0, freq=1.0,
                    space_discretization_type="galerkin", sdfem_type=2, delta0=1.0, delta1=1.0,
                    cell_measure=0, problem_linear=0, neumann_mask=0, poly_degree=0,
                    b_grad=None, t=0.0, ic=(0.0, 0.0, 0.0, 1.0), time_step=0.0,
                    time_discretization="crank_nicolson", bdf_two_first_step="backward_euler"):
    """b_grad: 3x3 gradient of a convection field linear in x (row-major).
    time_discretization: "crank_nicolson", "backward_euler" or "bdf_two";
    bdf_two_first_step: "backward_euler" or "crank_nicolson"."""
    a = AssemblyParams()
    if time_discretization not in TIME_SCHEMES:
        raise ValueError("time discretization scheme %r is not supported" % (time_discretization,))
    if bdf_two_first_step not in ("backward_euler", "crank_nicolson"):
        raise ValueError("bdf_two_first_step %r" % (bdf_two_first_step,))
    a.time_discretization = TIME_SCHEMES[time_discretization]
    a.bdf_two_first_step = 1 if bdf_two_first_step == "crank_nicolson" else 0
    if b_grad is not None:
        g = np.asarray(b_grad, dtype=np.float64).reshape(-1)
        for i in range(9):
            a.b_grad[i] = g[i]
    a.t = t
    a.time_step = time_step
    for i in range(4):
        a.ic[i] = ic[i]
    a.example, a.eps = example, eps
    for i in range(3):
        a.b[i] = b[i] if i < len(b) else 0.0
    a.c, a.freq = c, freq
    a.supg = 1 if space_discretization_type == "supg" else 0
    a.sdfem_type, a.delta0, a.delta1 = sdfem_type, delta0, delta1
    a.cell_measure, a.problem_linear = cell_measure, problem_linear
    a.neumann_mask, a.poly_degree = neumann_mask, poly_degree
    return a


def solver_params(preconditioner="jacobi", max_n_iterations=100, min_n_iterations=0,
                  gmres_restart=20, residual_tolerance=1e-8, residual_reduction=0.0,
                  divergence_factor=1e10, multigrid_n_levels=2, multigrid_cycle_type="V",
                  multigrid_n_pre_smooth=1, multigrid_n_post_smooth=1, jacobi_damp=1.0,
                  multigrid_correction_damp_factor=1.0, multigrid_smoother_coarse="direct_solve",
                  multigrid_coarse_residual=0.1, multigrid_coarse_max_n_iterations=10,
                  precision="fp64", gram_schmidt="classical"):
    """Defaults are the reference's database defaults."""
    s = SolverParams()
    s.preconditioner = {"no_preconditioner": 0, "jacobi": 1, "multigrid": 2}[preconditioner]
    s.max_n_iterations, s.min_n_iterations = max_n_iterations, min_n_iterations
    s.gmres_restart = gmres_restart
    s.residual_tolerance, s.residual_reduction = residual_tolerance, residual_reduction
    s.divergence_factor = divergence_factor
    s.multigrid_n_levels = multigrid_n_levels
    s.multigrid_cycle_type = {"V": 0, "W": 1, "F": 2}[multigrid_cycle_type]
    s.multigrid_n_pre_smooth, s.multigrid_n_post_smooth = multigrid_n_pre_smooth, multigrid_n_post_smooth
    s.jacobi_damp = jacobi_damp
    s.multigrid_correction_damp_factor = multigrid_correction_damp_factor
    s.multigrid_smoother_coarse = {"direct_solve": 0, "jacobi": 1}[multigrid_smoother_coarse]
    s.multigrid_coarse_residual = multigrid_coarse_residual
    s.multigrid_coarse_max_n_iterations = multigrid_coarse_max_n_iterations
    s.precision = {"fp64": 0, "mixed": 1}[precision]
    s.gram_schmidt = {"classical": 0, "modified": 1}[gram_schmidt]
    return s


class Hierarchy:
    """Host setup: unit square/cube (roots^dim cells) refined nref times, the
    Q_order space and CSR pattern of each of n_levels levels (0 = finest).
    tetra=True: roots^3 cubes of 6 Kuhn tetrahedra, P_order.  perturb > 0:
    the finest interior vertices moved by up to perturb*h (seeded); on
    quadrilaterals and hexahedra the cells become general (bilinear /
    trilinear maps).  ctx: number the DOFs
    and build the patterns on that context's GPU instead of the host."""

    def __init__(self, dim, order, nref, n_levels=1, roots=1, neumann_mask=0, tetra=False,
                 perturb=0.0, seed=0, ctx=None):
        self.dim, self.order, self.nref, self.n_levels = dim, order, nref, n_levels
        self.tetra = tetra
        h = ctypes.c_void_p()
        if tetra and ctx is not None:
            _chk(lib().cdg_hierarchy_create_tetra_device(ctx.c, order, roots, nref, n_levels,
                                                         neumann_mask, perturb, seed,
                                                         ctypes.byref(h)))
        elif tetra:
            _chk(lib().cdg_hierarchy_create_tetra(order, roots, nref, n_levels, neumann_mask,
                                                  perturb, seed, ctypes.byref(h)))
        elif ctx is not None:
            _chk(lib().cdg_hierarchy_create_device(ctx.c, dim, order, roots, nref, n_levels,
                                                   neumann_mask, ctypes.byref(h)))
        else:
            _chk(lib().cdg_hierarchy_create(dim, order, roots, nref, n_levels, neumann_mask,
                                            ctypes.byref(h)))
        self.h = h
        if not tetra and perturb > 0:
            # general quadrilaterals / hexahedra on the finest level
            _chk(lib().cdg_hierarchy_perturb(h, perturb, seed))

    def __del__(self):
        if getattr(self, "h", None):
            lib().cdg_hierarchy_destroy(self.h)
            self.h = None

    def info(self, level=0):
        a = np.zeros(6, dtype=np.int32)
        _chk(lib().cdg_hierarchy_level_info(self.h, level, _ip(a)))
        return dict(ncells=int(a[0]), nloc=int(a[1]), ndof=int(a[2]), nactive=int(a[3]),
                    nnz=int(a[4]), nv=int(a[5]))

    def mesh(self, level=0):
        i = self.info(level)
        v = np.zeros((i["ncells"], i["nv"], self.dim))
        _chk(lib().cdg_hierarchy_get_mesh(self.h, level, _dp(v)))
        return v

    def dofs(self, level=0):
        i = self.info(level)
        g = np.zeros((i["ncells"], i["nloc"]), dtype=np.int32)
        _chk(lib().cdg_hierarchy_get_dofs(self.h, level, _ip(g)))
        return g

    def pattern(self, level=0):
        i = self.info(level)
        rp = np.zeros(i["ndof"] + 1, dtype=np.int32)
        col = np.zeros(i["nnz"], dtype=np.int32)
        _chk(lib().cdg_hierarchy_get_pattern(self.h, level, _ip(rp), _ip(col)))
        return rp, col


def write_vector(filename, v):
    """BlockVector::write_to_file format: count line, raw doubles."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    _chk(lib().cdg_vector_write_file(os.fsencode(filename), _dp(v), v.size))


def read_vector(filename, n=0, capacity=None):
    """BlockVector::read_from_file: n > 0 requires that many entries."""
    cap = n if n > 0 else (capacity if capacity is not None else os.path.getsize(filename) // 8)
    v = np.zeros(max(cap, 1))
    got = ctypes.c_longlong(0)
    _chk(lib().cdg_vector_read_file(os.fsencode(filename), _dp(v), cap, n, ctypes.byref(got)))
    return v[:got.value].copy()


def checkpoint_file_name(base, time, overwrite=False):
    buf = ctypes.create_string_buffer(len(base) + 64)
    _chk(lib().cdg_checkpoint_file_name(os.fsencode(base), time, int(overwrite), buf,
                                        len(buf)))
    return buf.value.decode()


def space_number_device(ctx, cell_type, order, verts, neumann_mask=0):
    """TFESpace numbering on the GPU: (gdof[ncells, nloc], ndof, nactive)."""
    verts = np.ascontiguousarray(verts, dtype=np.float64)
    nv = 8 if cell_type == CELL_HEXA else 4
    dim = 2 if cell_type == CELL_QUAD else 3
    ncells = verts.size // (nv * dim)
    nloc = {(CELL_QUAD, 1): 4, (CELL_QUAD, 2): 9, (CELL_HEXA, 1): 8, (CELL_HEXA, 2): 27,
            (CELL_TETRA, 1): 4, (CELL_TETRA, 2): 10}[(cell_type, order)]
    g = np.zeros((ncells, nloc), dtype=np.int32)
    nd = ctypes.c_int(0)
    na = ctypes.c_int(0)
    _chk(lib().cdg_space_number_device(ctx.c, cell_type, order, neumann_mask, ncells, _dp(verts),
                                       _ip(g), ctypes.byref(nd), ctypes.byref(na)))
    return g, nd.value, na.value


def structure_build_device(ctx, gdof, ndof):
    """TStructure on the GPU: (row_ptr, col)."""
    gdof = np.ascontiguousarray(gdof, dtype=np.int32)
    ncells, nloc = gdof.shape
    rp = np.zeros(ndof + 1, dtype=np.int32)
    nnz = ctypes.c_longlong(0)
    cap = ncells * nloc * nloc
    col = np.zeros(cap, dtype=np.int32)
    _chk(lib().cdg_structure_build_device(ctx.c, ncells, nloc, ndof, _ip(gdof), _ip(rp), _ip(col),
                                          cap, ctypes.byref(nnz)))
    return rp, col[:nnz.value].copy()


class Context:
    """One CUDA device and stream."""

    def __init__(self, device=0):
        c = ctypes.c_void_p()
        _chk(lib().cdg_context_create(device, ctypes.byref(c)))
        self.c = c
        self.device = device
        self._problems = weakref.WeakSet()   # destroyed before the context

    def synchronize(self):
        _chk(lib().cdg_context_synchronize(self.c))

    def launches(self):
        return int(lib().cdg_context_launch_count(self.c))

    def stream(self):
        """The library's cudaStream_t as an integer handle."""
        s = ctypes.c_void_p()
        _chk(lib().cdg_context_stream(self.c, ctypes.byref(s)))
        return int(s.value or 0)

    def close(self):
        if getattr(self, "c", None):
            for p in list(getattr(self, "_problems", ())):
                p.close()
            lib().cdg_context_destroy(self.c)
            self.c = None

    def __del__(self):
        self.close()


class TimeErrors:
    """Errors integrated over time, as TimeConvectionDiffusion::output
    accumulates them (src/System/TimeConvectionDiffusion.C:936-966) and
    get_errors returns them (:1179-1187): the trapezoidal rule in time for
    L2(0,t;L2), L2(0,t;H1) (and L2(0,t;SUPG)), maxima for L_inf(0,t;L_inf) and
    L_inf(0,t;L2).  The previous value starts at zero, so the first add()
    counts half a step of the first error only."""

    def __init__(self, supg=False):
        self.supg = supg
        self.errors = [0.0] * 8
        self.t_linf = self.t_l2 = 0.0

    def add(self, local, tau, t):
        """local: ConvectionDiffusion.errors() at time t (L2, H1-semi, SD, DG, L_inf)."""
        e = self.errors
        e[0] += (local[0] * local[0] + e[1] * e[1]) * tau * 0.5
        e[1] = local[0]
        e[2] += (local[1] * local[1] + e[3] * e[3]) * tau * 0.5
        e[3] = local[1]
        if self.supg:
            e[6] += (local[2] * local[2] + e[7] * e[7]) * tau * 0.5
            e[7] = local[2]
        if e[4] < local[4]:
            e[4] = local[4]
            self.t_linf = t
        if e[5] < local[0]:
            e[5] = local[0]
            self.t_l2 = t

    def get_errors(self):
        """(L2(0,t;L2), L2(0,t;H1), L_inf(0,t;L_inf))"""
        return (float(np.sqrt(self.errors[0])), float(np.sqrt(self.errors[2])), self.errors[4])


class ConvectionDiffusion:
    """ConvectionDiffusion<d> on the GPU: one hierarchy's levels resident in HBM."""

    def __init__(self, ctx, hierarchy):
        self.ctx, self.hier = ctx, hierarchy
        p = ctypes.c_void_p()
        _chk(lib().cdg_problem_create(ctx.c, hierarchy.h, ctypes.byref(p)))
        self.p = p
        self.n_levels = hierarchy.n_levels
        self.dim = hierarchy.dim
        ctx._problems.add(self)

    @classmethod
    def from_arrays(cls, ctx, cell_type, order, levels):
        """cell_type: CELL_QUAD (2), CELL_HEXA (3), CELL_TETRA (4); levels:
        list (finest first) of dicts with verts (ncells,nv,dim), dofs
        (ncells,nloc), ndof, nactive, row_ptr, col, optional parent."""
        self = cls.__new__(cls)
        self.ctx, self.hier, self.n_levels = ctx, None, len(levels)
        self.dim = 2 if cell_type == CELL_QUAD else 3
        n = len(levels)
        keep = []

        def arr(dtype, key):
            out = (ctypes.c_void_p * n)()
            for i, l in enumerate(levels):
                if key in l and l[key] is not None:
                    a = np.ascontiguousarray(l[key], dtype=dtype)
                    keep.append(a)
                    out[i] = a.ctypes.data
            return out
        ncells = np.array([len(l["dofs"]) for l in levels], dtype=np.int32)
        ndof = np.array([l["ndof"] for l in levels], dtype=np.int32)
        nact = np.array([l["nactive"] for l in levels], dtype=np.int32)
        p = ctypes.c_void_p()
        _chk(lib().cdg_problem_create_from_arrays(
            ctx.c, cell_type, order, n, _ip(ncells), arr(np.float64, "verts"), arr(np.int32, "dofs"),
            _ip(ndof), _ip(nact), arr(np.int32, "row_ptr"), arr(np.int32, "col"),
            arr(np.int32, "parent"), ctypes.byref(p)))
        self.p = p
        ctx._problems.add(self)
        return self

    def close(self):
        if getattr(self, "p", None):
            if getattr(self.ctx, "c", None):
                lib().cdg_problem_destroy(self.p)
            self.p = None

    def __del__(self):
        self.close()

    def info(self, level=0):
        a = np.zeros(6, dtype=np.int32)
        _chk(lib().cdg_problem_level_info(self.p, level, _ip(a)))
        return dict(ncells=int(a[0]), nloc=int(a[1]), ndof=int(a[2]), nactive=int(a[3]),
                    nnz=int(a[4]), nv=int(a[5]))

    def write_solution(self, filename):
        _chk(lib().cdg_problem_write_solution(self.p, os.fsencode(filename)))

    def read_solution(self, filename):
        _chk(lib().cdg_problem_read_solution(self.p, os.fsencode(filename)))

    def checkpoint(self, base, step, time, every_n_steps=1, overwrite=False):
        """CheckpointIO::write(solution, time_stepping_scheme); True if written."""
        w = np.zeros(1, dtype=np.int32)
        _chk(lib().cdg_problem_checkpoint(self.p, os.fsencode(base), step, time, every_n_steps,
                                          int(overwrite), _ip(w)))
        return bool(w[0])

    def operator_layout(self, level=0):
        """lanes 0: CSR FP64 operator; else sliced ELLPACK with `lanes` lanes
        per row.  smoother_chunk 0: FP32 smoother streams CSR through
        registers; else entries per chunk staged through shared memory."""
        g = ctypes.c_int(0)
        t = ctypes.c_longlong(0)
        c = ctypes.c_int(0)
        _chk(lib().cdg_problem_operator_layout(self.p, level, ctypes.byref(g), ctypes.byref(t),
                                               ctypes.byref(c)))
        return dict(lanes=g.value, slots=t.value, smoother_chunk=c.value)

    def lattice(self, level=0):
        """dims: the DOF lattice of a uniform Q2 hexahedral level (zeros where
        there is none); transfer: the grid transfer to the next coarser level
        (-1 undecided, 0 CSR matrices, 1 lattice kernels)."""
        d = (ctypes.c_int * 3)()
        t = ctypes.c_int(0)
        _chk(lib().cdg_problem_lattice(self.p, level, d, ctypes.byref(t)))
        return dict(dims=tuple(d), transfer=t.value)

    def assemble(self, a):
        _chk(lib().cdg_problem_assemble(self.p, ctypes.byref(a)))

    def solve(self, s):
        st = SolveStats()
        _chk(lib().cdg_problem_solve(self.p, ctypes.byref(s), ctypes.byref(st)))
        return st

    def assemble_solve(self, a, s, solution_in=None, rhs_out=None, solution_out=None):
        st = SolveStats()
        nul = ctypes.POINTER(ctypes.c_double)()
        _chk(lib().cdg_problem_assemble_solve(
            self.p, ctypes.byref(a), ctypes.byref(s),
            _dp(solution_in) if solution_in is not None else nul,
            _dp(rhs_out) if rhs_out is not None else nul,
            _dp(solution_out) if solution_out is not None else nul, ctypes.byref(st)))
        return st

    def errors(self, a):
        e = np.zeros(5)
        _chk(lib().cdg_problem_errors(self.p, ctypes.byref(a), _dp(e)))
        return e

    # time-dependent CD (Crank-Nicolson)
    def tcd_initialize(self, a):
        _chk(lib().cdg_problem_tcd_initialize(self.p, ctypes.byref(a)))

    def tcd_step(self, a, tau, s):
        st = SolveStats()
        _chk(lib().cdg_problem_tcd_step(self.p, ctypes.byref(a), tau, ctypes.byref(s),
                                        ctypes.byref(st)))
        return st

    def tcd_matrix(self, which, level=0):
        """which: 0 stiffness, 1 mass, 2 system."""
        v = np.zeros(self.info(level)["nnz"])
        _chk(lib().cdg_problem_get_tcd_matrix(self.p, level, which, _dp(v)))
        return v

    def matrix(self, level=0):
        v = np.zeros(self.info(level)["nnz"])
        _chk(lib().cdg_problem_get_matrix(self.p, level, _dp(v)))
        return v

    def rhs(self, level=0):
        v = np.zeros(self.info(level)["ndof"])
        _chk(lib().cdg_problem_get_rhs(self.p, level, _dp(v)))
        return v

    def solution(self):
        v = np.zeros(self.info(0)["ndof"])
        _chk(lib().cdg_problem_get_solution(self.p, _dp(v)))
        return v

    def set_solution(self, x):
        """Host vector, or None to zero the solution on the device."""
        if x is None:
            _chk(lib().cdg_problem_set_solution(self.p, ctypes.POINTER(ctypes.c_double)()))
            return
        x = np.ascontiguousarray(x, dtype=np.float64)
        _chk(lib().cdg_problem_set_solution(self.p, _dp(x)))

    def slots(self, level=0):
        i = self.info(level)
        s = np.zeros((i["ncells"], i["nloc"] * i["nloc"]), dtype=np.int32)
        _chk(lib().cdg_problem_get_slots(self.p, level, _ip(s)))
        return s

    def apply(self, x, level=0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        _chk(lib().cdg_problem_apply(self.p, level, _dp(x), _dp(y)))
        return y

    def quadrature_points(self, a, level=0):
        """(ncells, nqp, dim): physical quadrature points of a level, where the
        caller evaluates its coefficient function"""
        nq = ctypes.c_int(0)
        _chk(lib().cdg_problem_quadrature_points(self.p, ctypes.byref(a), level,
                                                 ctypes.byref(nq), None))
        i = self.info(level)
        x = np.zeros((i["ncells"], nq.value, self.dim))
        _chk(lib().cdg_problem_quadrature_points(self.p, ctypes.byref(a), level,
                                                 ctypes.byref(nq), _dp(x)))
        return x

    def assemble_coefficients(self, a, level, coeffs):
        """assemble one level from coeffs (ncells, nqp, dim + 3): eps, b, c, f
        at every quadrature point (the reference's CoeffFct output)"""
        co = np.ascontiguousarray(coeffs, dtype=np.float64)
        _chk(lib().cdg_problem_assemble_coefficients(self.p, ctypes.byref(a), level, _dp(co)))

    def set_fp32_tensor_levels(self, enable=True):
        """levels between the finest and the coarsest assembled FP32-only by
        the tensor-core contraction (their FP64 values formed on demand)"""
        _chk(lib().cdg_problem_set_fp32_tensor_levels(self.p, 1 if enable else 0))

    def matrix32(self, level=0):
        v = np.zeros(self.info(level)["nnz"], dtype=np.float32)
        _chk(lib().cdg_problem_get_matrix32(self.p, level,
                                            v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return v

    def tuning(self, level=0):
        """(choice, (ms_csr, ms_matfree)): the FP32 multigrid kernel of a
        level (-2 not tuned yet, -1 CSR without a matrix-free operator, 0 CSR,
        1 matrix-free) and the tuner's best times of both kinds."""
        c, ms = self.tuning_detail(level)[:2]
        return c, ms

    def tuning_detail(self, level=0):
        """(choice, (ms_csr, ms_matfree), (csr_lanes_per_row, mf_blocks_per_sm))"""
        c = ctypes.c_int(0)
        sh = np.zeros(2, dtype=np.int32)
        ms = np.zeros(2)
        _chk(lib().cdg_problem_tuning(self.p, level, ctypes.byref(c), _ip(sh), _dp(ms)))
        return c.value, (float(ms[0]), float(ms[1])), (int(sh[0]), int(sh[1]))

    def apply32(self, x, level=0, variant=0):
        """y = A x with the FP32 multigrid operator of a level: variant 0 the
        CSR kernel, 1 the matrix-free kernel (Q2 hexahedra; one launch on
        uniform levels), 2 the two-launch matrix-free product, 3 the lattice
        stencil sweep (uniform Q2 lattices with Dirichlet data on the whole
        boundary)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros_like(x)
        fp = ctypes.POINTER(ctypes.c_float)
        _chk(lib().cdg_problem_apply32(self.p, level, variant, x.ctypes.data_as(fp),
                                       y.ctypes.data_as(fp)))
        return y

    def prolongate(self, xc, fine_level=0):
        xc = np.ascontiguousarray(xc, dtype=np.float64)
        xf = np.zeros(self.info(fine_level)["ndof"])
        _chk(lib().cdg_problem_prolongate(self.p, fine_level, _dp(xc), _dp(xf)))
        return xf

    def restrict(self, df, fine_level=0):
        df = np.ascontiguousarray(df, dtype=np.float64)
        rc = np.zeros(self.info(fine_level + 1)["ndof"])
        _chk(lib().cdg_problem_restrict(self.p, fine_level, _dp(df), _dp(rc)))
        return rc

    def time_kernel(self, kernel, a=None, level=0, reps=20):
        """Average ms per launch of a hot kernel (0 FP32 Jacobi smoothing step,
        1 FP64 SpMV, 2 element contraction + scatter, 3 FP32 defect)."""
        ms = np.zeros(1)
        _chk(lib().cdg_problem_time_kernel(self.p, ctypes.byref(a) if a is not None else None,
                                           kernel, level, reps, _dp(ms)))
        return float(ms[0])

    def precondition(self, s, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        z = np.zeros_like(v)
        _chk(lib().cdg_problem_precondition(self.p, ctypes.byref(s), _dp(v), _dp(z)))
        return z


# ---------------------------------------------------------------------------
# request server (served form: concurrent stationary solves on one GPU)
# ---------------------------------------------------------------------------
def request(dim, order, n, a, s):
    """A stationary CD solve on the unit square/cube with n cells per
    direction (n = roots * 2^k, roots 1 or 3); s.multigrid_n_levels <= 0 picks
    levels down to a 3- or 4-cell coarsest grid."""
    r = Request()
    r.dim, r.order, r.n, r.a, r.s = dim, order, n, a, s
    return r


def request_ndof(r):
    nd = ctypes.c_int()
    _chk(lib().cdg_request_ndof(ctypes.byref(r), ctypes.byref(nd)))
    return nd.value


def solve_batched(ctx, problems, params):
    """Solve assembled problems in one launch, one block per problem (the
    served form's batch): returns [(status, SolveStats)] in order.  params is
    one SolverParams for all or one per problem."""
    n = len(problems)
    if not isinstance(params, (list, tuple)):
        params = [params] * n
    arr = (ctypes.c_void_p * max(n, 1))(*[pr.p.value if hasattr(pr.p, "value") else pr.p
                                          for pr in problems])
    sp = (SolverParams * max(n, 1))(*params)
    st = (ctypes.c_int * max(n, 1))()
    stats = (SolveStats * max(n, 1))()
    _chk(lib().cdg_solve_batched(ctx.c, n, arr, sp, st, stats))
    return [(st[q], stats[q]) for q in range(n)]


class Server:
    """n_slots workers on one GPU; requests are admitted as slots free up and
    their problem instances fit the HBM budget (bytes; 0 = 80 % of free)."""

    COUNTERS = ("submitted", "completed", "failed", "queued", "running", "instances",
                "resident_bytes", "evictions", "budget_bytes", "peak_running", "launches",
                "classes")

    def __init__(self, device=0, n_slots=4, hbm_budget=0):
        h = ctypes.c_void_p()
        _chk(lib().cdg_server_create(device, n_slots, int(hbm_budget), ctypes.byref(h)))
        self.h = h
        self._out = {}

    def submit(self, r):
        """Queue a request; returns its ticket."""
        out = np.empty(request_ndof(r))
        t = ctypes.c_longlong()
        _chk(lib().cdg_server_submit(self.h, ctypes.byref(r), _dp(out), ctypes.byref(t)))
        self._out[t.value] = out
        return t.value

    def wait(self, ticket, timeout=-1.0):
        """(Result, solution) of a finished request, or None after the timeout."""
        res = Result()
        rc = lib().cdg_server_wait(self.h, ticket, timeout, ctypes.byref(res))
        if rc == 1:
            return None
        _chk(rc)
        return res, self._out.pop(ticket)

    def counters(self):
        c = (ctypes.c_longlong * 12)()
        _chk(lib().cdg_server_counters(self.h, c))
        b = (ctypes.c_longlong * 3)()
        _chk(lib().cdg_server_batch_counters(self.h, b))
        out = dict(zip(self.COUNTERS, list(c)))
        out.update(batch_launches=b[0], batched=b[1], batching=b[2])
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().cdg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
