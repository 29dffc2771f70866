"""ctypes binding of the CPU oracle (oracle/cd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The CUDA library never imports this.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcd_oracle.so")

(EX_SINE_LAPLACE, EX_SINE, EX_POLYEXP, EX_CONST_F, EX_POLY1, EX_BUMP, EX_POLY1_T, EX_EXP_SIN,
 EX_LINEAR_ST, EX_QUAD_ST) = range(10)
TIME_SCHEMES = {"crank_nicolson": 0, "backward_euler": 1, "bdf_two": 2}


class Config(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("order", ctypes.c_int), ("nref", ctypes.c_int),
        ("example", ctypes.c_int), ("eps", ctypes.c_double),
        ("b", ctypes.c_double * 3), ("c", ctypes.c_double),
        ("freq", ctypes.c_double), ("supg", ctypes.c_int),
        ("sdfem_type", ctypes.c_int), ("delta0", ctypes.c_double),
        ("delta1", ctypes.c_double), ("cell_measure", ctypes.c_int),
        ("problem_linear", ctypes.c_int), ("neumann_mask", ctypes.c_int),
        ("poly_degree", ctypes.c_int), ("tetra", ctypes.c_int),
        ("b_grad", ctypes.c_double * 9), ("t", ctypes.c_double),
        ("ic", ctypes.c_double * 4), ("time_step", ctypes.c_double),
        ("time_disc", ctypes.c_int), ("bdf_first", ctypes.c_int),
    ]


class SolverConfig(ctypes.Structure):
    _fields_ = [
        ("precond", ctypes.c_int), ("max_it", ctypes.c_int),
        ("min_it", ctypes.c_int), ("restart", ctypes.c_int),
        ("tol_abs", ctypes.c_double), ("reduction", ctypes.c_double),
        ("divergence", ctypes.c_double), ("mg_levels", ctypes.c_int),
        ("mg_cycle", ctypes.c_int), ("n_pre", ctypes.c_int),
        ("n_post", ctypes.c_int), ("jacobi_damp", ctypes.c_double),
        ("correction_damp", ctypes.c_double), ("coarse_direct", ctypes.c_int),
        ("coarse_eps", ctypes.c_double), ("coarse_maxit", ctypes.c_int),
        ("classical_gs", ctypes.c_int),
    ]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "cd_oracle.c")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(Config), ctypes.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_create_from_arrays.restype = P
        L.orc_create_from_arrays.argtypes = [
            ctypes.POINTER(Config), ctypes.c_int, ip, ctypes.POINTER(dp),
            ctypes.POINTER(ip), ip, ip, ctypes.POINTER(ip), ctypes.POINTER(ip)]
        L.orc_last_error.restype = ctypes.c_char_p
        for name, args in [
            ("orc_level_info", [P, ctypes.c_int, ip]),
            ("orc_get_mesh", [P, ctypes.c_int, dp]),
            ("orc_get_gdof", [P, ctypes.c_int, ip]),
            ("orc_get_structure", [P, ctypes.c_int, ip, ip]),
            ("orc_get_matrix", [P, ctypes.c_int, dp]),
            ("orc_get_rhs", [P, ctypes.c_int, dp]),
            ("orc_get_solution", [P, dp]),
            ("orc_set_solution", [P, dp]),
            ("orc_assemble", [P]),
            ("orc_local_system", [P, ctypes.c_int, ctypes.c_int, dp, dp]),
            ("orc_apply", [P, ctypes.c_int, dp, dp]),
            ("orc_prolongate", [P, ctypes.c_int, dp, dp]),
            ("orc_restrict", [P, ctypes.c_int, dp, dp]),
            ("orc_mg_apply", [P, ctypes.POINTER(SolverConfig), dp, dp]),
            ("orc_solve", [P, ctypes.POINTER(SolverConfig), ip, dp, dp]),
            ("orc_errors", [P, dp]),
            ("orc_tcd_initialize", [P]),
            ("orc_tcd_step", [P, ctypes.c_double, ctypes.c_double,
                              ctypes.POINTER(SolverConfig), ip, dp, dp]),
            ("orc_get_tcd_matrix", [P, ctypes.c_int, ctypes.c_int, dp]),
            ("orc_quadrature_points", [P, ctypes.c_int, ip, dp]),
            ("orc_assemble_coefficients", [P, ctypes.c_int, dp]),
            ("orc_marker_numbering", [ctypes.POINTER(Config), ctypes.c_int, dp, ip, ip, ip]),
        ]:
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def marker_numbering(cfg, verts):
    """The reference's marker-algorithm numbering (TFESpace3D::ConstructSpace,
    FESpace3D.C:186-420) of a tetrahedral mesh given as verts[cell, 4, 3]:
    (gdof[cell, nloc], ndof, nactive)."""
    v = np.ascontiguousarray(verts, dtype=np.float64)
    nc = v.shape[0]
    nloc = 4 if cfg.order == 1 else 10
    g = np.zeros((nc, nloc), dtype=np.int32)
    nd = ctypes.c_int(0)
    na = ctypes.c_int(0)
    if lib().orc_marker_numbering(ctypes.byref(cfg), nc, _dp(v), _ip(g), ctypes.byref(nd),
                                  ctypes.byref(na)):
        raise RuntimeError(lib().orc_last_error().decode())
    return g, nd.value, na.value


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def make_config(dim, order, nref, example, eps=1.0, b=(0, 0, 0), c=0.0, freq=1.0,
                supg=False, sdfem_type=2, delta0=1.0, delta1=1.0, cell_measure=0,
                problem_linear=0, neumann_mask=0, poly_degree=0, tetra=False,
                b_grad=None, t=0.0, ic=(0.5, 0.5, 0.5, 0.1), time_step=0.0,
                time_discretization="crank_nicolson", bdf_two_first_step="backward_euler"):
    cfg = Config()
    cfg.dim, cfg.order, cfg.nref, cfg.example = dim, order, nref, example
    cfg.eps = eps
    for i in range(3):
        cfg.b[i] = b[i] if i < len(b) else 0.0
    cfg.c, cfg.freq, cfg.supg = c, freq, int(supg)
    cfg.sdfem_type, cfg.delta0, cfg.delta1 = sdfem_type, delta0, delta1
    cfg.cell_measure, cfg.problem_linear = cell_measure, problem_linear
    cfg.neumann_mask, cfg.poly_degree = neumann_mask, poly_degree
    cfg.tetra = int(tetra)
    if b_grad is not None:
        bg = np.asarray(b_grad, dtype=np.float64).reshape(-1)
        for i in range(9):
            cfg.b_grad[i] = float(bg[i])
    cfg.t = t
    cfg.time_step = time_step
    cfg.time_disc = TIME_SCHEMES[time_discretization]
    cfg.bdf_first = 1 if bdf_two_first_step == "crank_nicolson" else 0
    for i in range(4):
        cfg.ic[i] = ic[i]
    return cfg


def make_solver(precond="jacobi", max_it=1000, min_it=0, restart=50, tol_abs=0.0,
                reduction=1e-10, divergence=1e10, mg_levels=2, mg_cycle="V",
                n_pre=2, n_post=2, jacobi_damp=1.0, correction_damp=1.0,
                coarse_direct=True, coarse_eps=0.1, coarse_maxit=10, gram_schmidt="classical"):
    s = SolverConfig()
    s.precond = {"none": 0, "jacobi": 1, "multigrid": 2}[precond]
    s.max_it, s.min_it, s.restart = max_it, min_it, restart
    s.tol_abs, s.reduction, s.divergence = tol_abs, reduction, divergence
    s.mg_levels = mg_levels
    s.mg_cycle = {"V": 0, "W": 1, "F": 2}[mg_cycle]
    s.n_pre, s.n_post = n_pre, n_post
    s.jacobi_damp, s.correction_damp = jacobi_damp, correction_damp
    s.coarse_direct, s.coarse_eps, s.coarse_maxit = int(coarse_direct), coarse_eps, coarse_maxit
    s.classical_gs = 1 if gram_schmidt == "classical" else 0
    return s


class Problem:
    """One CD problem on a hierarchy of uniformly refined grids (level 0 finest)."""

    def __init__(self, cfg, n_levels=1, arrays=None):
        """arrays: list (finest first) of dicts with verts (ncells, nv, dim),
        gdof (ncells, nloc), ndof, nactive, row_ptr, col -- the levels are
        taken as given (orc_create_from_arrays)."""
        self.cfg = cfg
        self.n_levels = n_levels
        if arrays is None:
            self.h = lib().orc_create(ctypes.byref(cfg), n_levels)
        else:
            n = len(arrays)
            self.n_levels = n
            keep = []
            ncells = np.array([a["gdof"].shape[0] for a in arrays], dtype=np.int32)
            ndof = np.array([a["ndof"] for a in arrays], dtype=np.int32)
            nact = np.array([a["nactive"] for a in arrays], dtype=np.int32)
            dp = ctypes.POINTER(ctypes.c_double)
            ipt = ctypes.POINTER(ctypes.c_int)
            vp, gp, rp, cp = (dp * n)(), (ipt * n)(), (ipt * n)(), (ipt * n)()
            for k, a in enumerate(arrays):
                v = np.ascontiguousarray(a["verts"], dtype=np.float64)
                g = np.ascontiguousarray(a["gdof"], dtype=np.int32)
                r = np.ascontiguousarray(a["row_ptr"], dtype=np.int32)
                c = np.ascontiguousarray(a["col"], dtype=np.int32)
                keep += [v, g, r, c]
                vp[k], gp[k], rp[k], cp[k] = _dp(v), _ip(g), _ip(r), _ip(c)
            self.h = lib().orc_create_from_arrays(ctypes.byref(cfg), n, _ip(ncells), vp, gp,
                                                  _ip(ndof), _ip(nact), rp, cp)
        if not self.h:
            raise RuntimeError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError(lib().orc_last_error().decode())

    def info(self, level=0):
        a = np.zeros(6, dtype=np.int32)
        self._chk(lib().orc_level_info(self.h, level, _ip(a)))
        return dict(ncells=int(a[0]), nloc=int(a[1]), ndof=int(a[2]), nactive=int(a[3]),
                    nnz=int(a[4]), nv=int(a[5]))

    def mesh(self, level=0):
        i = self.info(level)
        v = np.zeros((i["ncells"], i["nv"], self.cfg.dim))
        self._chk(lib().orc_get_mesh(self.h, level, _dp(v)))
        return v

    def gdof(self, level=0):
        i = self.info(level)
        g = np.zeros((i["ncells"], i["nloc"]), dtype=np.int32)
        self._chk(lib().orc_get_gdof(self.h, level, _ip(g)))
        return g

    def structure(self, level=0):
        i = self.info(level)
        rp = np.zeros(i["ndof"] + 1, dtype=np.int32)
        col = np.zeros(i["nnz"], dtype=np.int32)
        self._chk(lib().orc_get_structure(self.h, level, _ip(rp), _ip(col)))
        return rp, col

    def assemble(self):
        self._chk(lib().orc_assemble(self.h))

    def matrix(self, level=0):
        i = self.info(level)
        v = np.zeros(i["nnz"])
        self._chk(lib().orc_get_matrix(self.h, level, _dp(v)))
        return v

    def rhs(self, level=0):
        v = np.zeros(self.info(level)["ndof"])
        self._chk(lib().orc_get_rhs(self.h, level, _dp(v)))
        return v

    def solution(self):
        v = np.zeros(self.info(0)["ndof"])
        self._chk(lib().orc_get_solution(self.h, _dp(v)))
        return v

    def set_solution(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._chk(lib().orc_set_solution(self.h, _dp(x)))

    def local_system(self, cell, level=0):
        n = self.info(level)["nloc"]
        A = np.zeros((n, n))
        f = np.zeros(n)
        self._chk(lib().orc_local_system(self.h, level, cell, _dp(A), _dp(f)))
        return A, f

    def apply(self, x, level=0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._chk(lib().orc_apply(self.h, level, _dp(x), _dp(y)))
        return y

    def prolongate(self, xc, fine_level=0):
        xc = np.ascontiguousarray(xc, dtype=np.float64)
        xf = np.zeros(self.info(fine_level)["ndof"])
        self._chk(lib().orc_prolongate(self.h, fine_level, _dp(xc), _dp(xf)))
        return xf

    def restrict(self, df, fine_level=0):
        df = np.ascontiguousarray(df, dtype=np.float64)
        rc = np.zeros(self.info(fine_level + 1)["ndof"])
        self._chk(lib().orc_restrict(self.h, fine_level, _dp(df), _dp(rc)))
        return rc

    def mg_apply(self, scfg, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        z = np.zeros_like(v)
        self._chk(lib().orc_mg_apply(self.h, ctypes.byref(scfg), _dp(v), _dp(z)))
        return z

    def solve(self, scfg):
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        ini = np.zeros(1)
        self._chk(lib().orc_solve(self.h, ctypes.byref(scfg), _ip(it), _dp(res), _dp(ini)))
        return int(it[0]), float(res[0]), float(ini[0])

    def errors(self):
        e = np.zeros(5)
        self._chk(lib().orc_errors(self.h, _dp(e)))
        return e

    def quadrature_points(self, level=0):
        """(ncells, nqp, dim) physical quadrature points of a level"""
        nq = np.zeros(1, dtype=np.int32)
        self._chk(lib().orc_quadrature_points(self.h, level, _ip(nq), None))
        i = self.info(level)
        x = np.zeros((i["ncells"], int(nq[0]), self.cfg.dim))
        self._chk(lib().orc_quadrature_points(self.h, level, _ip(nq), _dp(x)))
        return x

    def assemble_coefficients(self, level, coeffs):
        """assemble one level with coeffs (ncells, nqp, dim + 3): eps, b, c, f
        per quadrature point"""
        co = np.ascontiguousarray(coeffs, dtype=np.float64)
        self._chk(lib().orc_assemble_coefficients(self.h, level, _dp(co)))

    def tcd_initialize(self):
        self._chk(lib().orc_tcd_initialize(self.h))

    def tcd_step(self, t_new, tau, scfg):
        it = np.zeros(1, dtype=np.int32)
        res = np.zeros(1)
        ini = np.zeros(1)
        self._chk(lib().orc_tcd_step(self.h, t_new, tau, ctypes.byref(scfg), _ip(it),
                                     _dp(res), _dp(ini)))
        return int(it[0]), float(res[0]), float(ini[0])

    def tcd_matrix(self, which, level=0):
        """which: 0 stiffness, 1 mass, 2 system"""
        v = np.zeros(self.info(level)["nnz"])
        self._chk(lib().orc_get_tcd_matrix(self.h, level, which, _dp(v)))
        return v
