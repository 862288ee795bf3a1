"""ctypes binding of libmrgpu (the C ABI in include/mrgpu.h).

This module is the Python-side host mirror of the foam-extend plug-in
boundary.  It loads the in-tree ``_lib/libmrgpu.so`` and fails loudly when the
library is missing or no CUDA device is present: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmrgpu.so")

MRG_OK, MRG_E_INVALID, MRG_E_OOM, MRG_E_BREAKDOWN, MRG_E_TIMEOUT, MRG_E_CUDA, MRG_E_BUSY = range(7)
SOLVERS = {"PCG": 0, "PBiCG": 1, "BiCGStab": 2, "smoothSolver": 3, "GAMG": 4}
SMOOTHERS = {"GaussSeidel": 0, "DIC": 1, "DILU": 2, "DICGaussSeidel": 3, "DILUGaussSeidel": 4}
PRECONDITIONERS = {"none": 0, "diagonal": 1, "DIC": 2, "DILU": 3, "block": 4}
PRECISIONS = {"fp64": 0, "mixed": 1}
ORDERINGS = {"exact": 0, "colour": 1}
AGGLOMERATORS = {"algebraicPair": 0, "faceAreaPair": 1}

EXPORTED = [
    "mrg_last_error", "mrg_version", "mrg_controls_default", "mrg_ctx_create", "mrg_ctx_destroy",
    "mrg_ctx_set_watchdog",
    "mrg_ctx_mem_used", "mrg_host_alloc", "mrg_host_free", "mrg_mesh_upload", "mrg_mesh_destroy",
    "mrg_mesh_levels", "mrg_mesh_set_face_areas", "mrg_mesh_set_blocks", "mrg_coeffs_upload", "mrg_coeffs_upload_device", "mrg_solve", "mrg_solve_device",
    "mrg_amul", "mrg_residual", "mrg_precondition", "mrg_factor_diag", "mrg_ggi_create", "mrg_ggi_destroy",
    "mrg_ggi_apply", "mrg_ggi_apply_device", "mrg_ggi_time", "mrg_ggi_build", "mrg_direct_map_build", "mrg_ggi_get", "mrg_dev_alloc", "mrg_dev_free", "mrg_dev_copy",
    "mrg_event_record", "mrg_event_elapsed", "mrg_kernel_launches", "mrg_time_kernel",
    "mrg_batch_create", "mrg_batch_destroy", "mrg_batch_solve", "mrg_batch_solve_device",
    "mrg_residual_noalloc", "mrg_server_create", "mrg_server_destroy", "mrg_server_submit", "mrg_server_poll",
    "mrg_server_wait", "mrg_server_get_stats", "mrg_mesh_tune", "mrg_batch_tune",
    "mrg_dn_create", "mrg_dn_destroy", "mrg_dn_set_state", "mrg_dn_new_time_step", "mrg_dn_update_jump",
    "mrg_dn_update_flux", "mrg_dn_rhs", "mrg_dn_residuals", "mrg_dn_get_state", "mrg_dn_criteria",
    "mrg_dn_set_flux_relaxation",
    "mrg_mono_create", "mrg_mono_destroy", "mrg_mono_update", "mrg_mono_source",
    "mrg_block_addressing", "mrg_block_coeffs",
]


class MrgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mrgpu error {code}: {msg}")
        self.code = code


class Controls(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("rel_tol", C.c_double), ("min_iter", C.c_int),
                ("max_iter", C.c_int), ("solver", C.c_int), ("preconditioner", C.c_int),
                ("precision", C.c_int), ("ordering", C.c_int), ("inner_rel_tol", C.c_double),
                ("inner_max_iter", C.c_int), ("max_outer", C.c_int), ("iters_per_launch", C.c_int),
                ("smoother", C.c_int), ("n_sweeps", C.c_int), ("gamg_coarsest_cells", C.c_int),
                ("gamg_post_sweeps", C.c_int), ("gamg_finest_sweeps", C.c_int),
                ("gamg_max_post_sweeps", C.c_int), ("gamg_post_sweeps_level_multiplier", C.c_int),
                ("gamg_scale_correction", C.c_int), ("gamg_agglomerator", C.c_int)]


class Perf(C.Structure):
    _fields_ = [("initial_residual", C.c_double), ("final_residual", C.c_double), ("n_iter", C.c_int),
                ("converged", C.c_int), ("singular", C.c_int), ("status", C.c_int), ("n_outer", C.c_int),
                ("fallback", C.c_int), ("solve_ms", C.c_double)]

    def as_dict(self):
        return {"initial_residual": self.initial_residual, "final_residual": self.final_residual,
                "n_iter": self.n_iter, "converged": bool(self.converged), "singular": bool(self.singular),
                "status": self.status, "n_outer": self.n_outer, "fallback": bool(self.fallback),
                "solve_ms": self.solve_ms}


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("running", C.c_int), ("queued", C.c_int),
                ("peak_running", C.c_int), ("reserved", C.c_int), ("inflight_bytes", C.c_size_t),
                ("peak_inflight_bytes", C.c_size_t)]


class Tuning(C.Structure):
    _fields_ = [("mode", C.c_int), ("iters_per_launch", C.c_int), ("sweep_chunks_per_cta", C.c_int),
                ("spmv_kernel", C.c_int), ("spmv_block_threads", C.c_int), ("spmv_rows_per_warp_step", C.c_int),
                ("candidates", C.c_int), ("reserved", C.c_int), ("us_per_iter", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MonoPatch(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("face_cells", C.c_void_p), ("weights", C.c_void_p),
                ("mag_long_delta", C.c_void_p), ("delta_coeffs", C.c_void_p), ("mag_sf", C.c_void_p),
                ("src_ptr", C.c_void_p), ("src_face", C.c_void_p), ("src_weight", C.c_void_p)]


class DnPatch(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("face_cells", C.c_void_p),
                ("delta_coeffs", C.c_void_p), ("k", C.c_void_p), ("area", C.c_void_p), ("src_ptr", C.c_void_p),
                ("src_face", C.c_void_p), ("src_weight", C.c_void_p)]


class DnConfig(C.Structure):
    _fields_ = [("K", C.c_double), ("flux_jump", C.c_double), ("relax", C.c_double), ("relax_model", C.c_int),
                ("coupling_reuse", C.c_int)]


class IfaceDesc(C.Structure):
    _fields_ = [("n_faces", C.c_int), ("face_cells", C.POINTER(C.c_int32)), ("src_ptr", C.POINTER(C.c_int32)),
                ("src_cell", C.POINTER(C.c_int32)), ("src_weight", C.POINTER(C.c_double))]


_LIB = None


def load(path: str = LIB_PATH):
    """Load libmrgpu; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libmrgpu not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    L.mrg_last_error.restype = C.c_char_p
    L.mrg_version.restype = C.c_char_p
    L.mrg_controls_default.argtypes = [C.POINTER(Controls)]
    L.mrg_ctx_create.argtypes = [C.c_int, C.c_size_t, C.POINTER(vp)]
    L.mrg_ctx_destroy.argtypes = [vp]
    L.mrg_ctx_mem_used.argtypes = [vp, C.POINTER(C.c_size_t)]
    L.mrg_ctx_set_watchdog.argtypes = [vp, C.c_longlong, C.c_int]
    L.mrg_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
    L.mrg_host_free.argtypes = [vp]
    L.mrg_mesh_upload.argtypes = [vp, C.c_int, C.c_int, ip, ip, C.c_int, C.POINTER(IfaceDesc), C.POINTER(vp)]
    L.mrg_mesh_destroy.argtypes = [vp]
    L.mrg_mesh_levels.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.mrg_mesh_set_face_areas.argtypes = [vp, dp]
    L.mrg_mesh_set_blocks.argtypes = [vp, C.c_int, C.c_int, C.c_int, ip, ip]
    L.mrg_coeffs_upload.argtypes = [vp, dp, dp, dp, dp, dp]
    L.mrg_coeffs_upload_device.argtypes = [vp, vp, vp, vp, vp, vp]
    L.mrg_solve.argtypes = [vp, dp, dp, C.POINTER(Controls), C.POINTER(Perf)]
    L.mrg_solve_device.argtypes = [vp, vp, vp, C.POINTER(Controls), C.POINTER(Perf)]
    L.mrg_amul.argtypes = [vp, dp, dp, C.c_int]
    L.mrg_residual.argtypes = [vp, dp, dp, dp, dp]
    L.mrg_precondition.argtypes = [vp, C.c_int, C.c_int, dp, dp, C.c_int]
    L.mrg_factor_diag.argtypes = [vp, C.c_int, C.c_int, dp]
    L.mrg_ggi_create.argtypes = [vp, C.c_int, C.c_int, ip, ip, dp, C.POINTER(vp)]
    L.mrg_ggi_destroy.argtypes = [vp]
    L.mrg_ggi_apply.argtypes = [vp, dp, dp, C.c_int]
    L.mrg_ggi_apply_device.argtypes = [vp, vp, vp, C.c_int]
    L.mrg_ggi_time.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.mrg_ggi_build.argtypes = [vp, C.c_int, ip, dp, C.c_int, ip, dp, C.c_double, C.POINTER(vp), C.POINTER(vp)]
    L.mrg_direct_map_build.argtypes = [vp, C.c_int, dp, C.c_int, dp, C.c_double, C.POINTER(vp), C.POINTER(vp)]
    ipp = C.POINTER(C.c_int)
    L.mrg_ggi_get.argtypes = [vp, ipp, ipp, ipp, ip, ip, dp]
    L.mrg_dev_alloc.argtypes = [vp, C.c_size_t, C.POINTER(vp)]
    L.mrg_dev_free.argtypes = [vp, vp]
    L.mrg_dev_copy.argtypes = [vp, vp, vp, C.c_size_t, C.c_int]
    L.mrg_event_record.argtypes = [vp, C.c_int]
    L.mrg_event_elapsed.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.mrg_kernel_launches.argtypes = [C.POINTER(C.c_uint64)]
    L.mrg_time_kernel.argtypes = [vp, C.POINTER(Controls), C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.mrg_batch_create.argtypes = [vp, C.c_int, C.POINTER(vp), C.c_int, C.POINTER(vp)]
    L.mrg_batch_destroy.argtypes = [vp]
    L.mrg_batch_solve.argtypes = [vp, C.POINTER(dp), C.POINTER(dp), C.POINTER(Controls), C.POINTER(Perf)]
    L.mrg_batch_solve_device.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(Controls), C.POINTER(Perf)]
    L.mrg_residual_noalloc.argtypes = [C.c_int, C.c_int] + [vp] * 11 + [dp, dp]
    L.mrg_server_create.argtypes = [vp, C.POINTER(Controls), C.POINTER(Controls), C.c_size_t, C.c_int,
                                    C.POINTER(vp)]
    L.mrg_server_destroy.argtypes = [vp]
    L.mrg_server_submit.argtypes = [vp, vp, C.c_int] + [vp] * 8 + [C.POINTER(C.c_uint64)]
    L.mrg_server_poll.argtypes = [vp, C.c_uint64, C.POINTER(C.c_int), C.POINTER(Perf), C.POINTER(C.c_double)]
    L.mrg_server_wait.argtypes = [vp, C.c_uint64, C.c_double, C.POINTER(C.c_int), C.POINTER(Perf),
                                  C.POINTER(C.c_double)]
    L.mrg_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
    L.mrg_mesh_tune.argtypes = [vp, vp, vp, C.POINTER(Controls), C.POINTER(Tuning)]
    L.mrg_dn_create.argtypes = [vp, C.POINTER(DnPatch), C.POINTER(DnPatch), C.POINTER(DnConfig), C.POINTER(vp)]
    L.mrg_dn_destroy.argtypes = [vp]
    L.mrg_dn_set_state.argtypes = [vp, dp, dp]
    L.mrg_dn_set_flux_relaxation.argtypes = [vp, C.c_int, C.c_double, C.c_int]
    L.mrg_dn_new_time_step.argtypes = [vp]
    L.mrg_dn_update_jump.argtypes = [vp, vp]
    L.mrg_dn_update_flux.argtypes = [vp, vp]
    L.mrg_dn_rhs.argtypes = [vp, C.c_int, vp, vp]
    L.mrg_dn_residuals.argtypes = [vp, vp, vp, dp, dp]
    L.mrg_dn_get_state.argtypes = [vp, dp, dp, dp]
    L.mrg_dn_criteria.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
    L.mrg_mono_create.argtypes = [vp, C.POINTER(MonoPatch), C.POINTER(MonoPatch), C.POINTER(vp)]
    L.mrg_mono_destroy.argtypes = [vp]
    L.mrg_mono_update.argtypes = [vp, C.c_int] + [vp] * 8
    L.mrg_mono_source.argtypes = [vp, C.c_int] + [vp] * 6
    L.mrg_batch_tune.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(Controls), C.POINTER(Tuning)]
    L.mrg_block_addressing.argtypes = [C.c_int, C.c_int, ip, ip, C.c_int, C.POINTER(C.c_int), ip, ip]
    L.mrg_block_coeffs.argtypes = [C.c_int, C.c_int, ip, ip, C.c_int, dp, dp, dp, dp, dp, dp]
    _LIB = L
    return L


def _check(rc):
    if rc != MRG_OK:
        raise MrgError(rc, load().mrg_last_error().decode())


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


def controls(tol=1e-6, rel_tol=0.0, min_iter=0, max_iter=1000, solver="PCG", precond="DIC",
             precision="fp64", ordering="exact", inner_rel_tol=1e-5, inner_max_iter=0, max_outer=50,
             iters_per_launch=16, n_sweeps=1, smoother="GaussSeidel", n_coarsest_cells=10, n_post_sweeps=2,
             n_finest_sweeps=2, max_post_sweeps=4, post_sweeps_level_multiplier=1, scale_correction=True,
             agglomerator="algebraicPair") -> Controls:
    c = Controls()
    load().mrg_controls_default(C.byref(c))
    c.tolerance, c.rel_tol, c.min_iter, c.max_iter = tol, rel_tol, min_iter, max_iter
    c.solver, c.preconditioner = SOLVERS[solver], PRECONDITIONERS[precond]
    c.precision, c.ordering = PRECISIONS[precision], ORDERINGS[ordering]
    c.inner_rel_tol, c.inner_max_iter, c.max_outer = inner_rel_tol, inner_max_iter, max_outer
    c.iters_per_launch = iters_per_launch
    c.smoother, c.n_sweeps = SMOOTHERS[smoother], n_sweeps
    c.gamg_coarsest_cells, c.gamg_post_sweeps, c.gamg_finest_sweeps = n_coarsest_cells, n_post_sweeps, n_finest_sweeps
    c.gamg_max_post_sweeps, c.gamg_post_sweeps_level_multiplier = max_post_sweeps, post_sweeps_level_multiplier
    c.gamg_scale_correction, c.gamg_agglomerator = int(bool(scale_correction)), AGGLOMERATORS[agglomerator]
    return c


class Context:
    """A device context (one CUDA stream, an HBM budget)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        L = load()
        h = C.c_void_p()
        _check(L.mrg_ctx_create(device, hbm_budget, C.byref(h)))
        self.h = h
        self._meshes = []

    def mem_used(self) -> int:
        v = C.c_size_t()
        _check(load().mrg_ctx_mem_used(self.h, C.byref(v)))
        return v.value

    # -- resident buffers and device timing (no foam counterpart) ----------
    def set_watchdog(self, wait_cycles: int = 0, unpublished_chunk: int = -1):
        """Budget of every device wait in SM cycles (0: the default, ~2 s) and
        the test hook that leaves one chunk of the exact forward sweep
        unpublished (-1: off); see mrg_ctx_set_watchdog."""
        _check(load().mrg_ctx_set_watchdog(self.h, int(wait_cycles), int(unpublished_chunk)))

    def dev_alloc(self, nbytes: int) -> int:
        p = C.c_void_p()
        _check(load().mrg_dev_alloc(self.h, nbytes, C.byref(p)))
        return p.value

    def dev_free(self, p: int):
        _check(load().mrg_dev_free(self.h, C.c_void_p(p)))

    def to_device(self, arr: np.ndarray) -> int:
        arr = np.ascontiguousarray(arr)
        p = self.dev_alloc(arr.nbytes)
        _check(load().mrg_dev_copy(self.h, C.c_void_p(p), arr.ctypes.data_as(C.c_void_p), arr.nbytes, 0))
        return p

    def from_device(self, p: int, out: np.ndarray) -> np.ndarray:
        _check(load().mrg_dev_copy(self.h, out.ctypes.data_as(C.c_void_p), C.c_void_p(p), out.nbytes, 1))
        return out

    def copy_d2d(self, dst: int, src: int, nbytes: int):
        _check(load().mrg_dev_copy(self.h, C.c_void_p(dst), C.c_void_p(src), nbytes, 2))

    def record(self, slot: int):
        _check(load().mrg_event_record(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_float()
        _check(load().mrg_event_elapsed(self.h, a, b, C.byref(v)))
        return v.value

    def close(self):
        for m in self._meshes:
            m.close()
        self._meshes = []
        if self.h:
            _check(load().mrg_ctx_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launches() -> int:
    v = C.c_uint64()
    _check(load().mrg_kernel_launches(C.byref(v)))
    return v.value


def residual_noalloc(n_cells: int, n_faces: int, d_lower_addr: int, d_upper_addr: int, d_owner_start: int,
                     d_losort: int, d_losort_start: int, d_diag: int, d_upper: int, d_lower: int | None,
                     d_b: int, d_x: int, stream: int | None = None) -> tuple[float, float]:
    """mrg_residual_noalloc on device arrays (integer device addresses):
    returns (residual, norm_factor) without allocating device memory."""
    r, nf = C.c_double(), C.c_double()
    _check(load().mrg_residual_noalloc(int(n_cells), int(n_faces), *[C.c_void_p(p) for p in (
        d_lower_addr, d_upper_addr, d_owner_start, d_losort, d_losort_start, d_diag, d_upper, d_lower, d_b, d_x,
        stream)], C.byref(r), C.byref(nf)))
    return r.value, nf.value


def host_array(ctx_unused, n: int, dtype=np.float64) -> np.ndarray:
    """A numpy array over pinned (page-locked) host memory."""
    nbytes = int(n) * np.dtype(dtype).itemsize
    p = C.c_void_p()
    _check(load().mrg_host_alloc(nbytes, C.byref(p)))
    buf = (C.c_char * nbytes).from_address(p.value)
    return np.frombuffer(buf, dtype=dtype, count=int(n))  # lives until process exit


class Mesh:
    """Resident LDU addressing (+ interface patches) on the device."""

    def __init__(self, ctx: Context, n, lower, upper, iface=None):
        L = load()
        self.ctx = ctx
        self.n = int(n)
        self._lower = np.ascontiguousarray(lower, dtype=np.int32)
        self._upper = np.ascontiguousarray(upper, dtype=np.int32)
        self.nf = len(self._lower)
        descs = None
        nif = 0
        self.ni = 0
        if iface is not None and len(iface["cells"]) > 0:
            self._if = {k: np.ascontiguousarray(iface[k], dtype=np.int32) for k in ("cells", "ptr", "src")}
            self._if["w"] = np.ascontiguousarray(iface["w"], dtype=np.float64)
            d = IfaceDesc()
            d.n_faces = len(self._if["cells"])
            d.face_cells, d.src_ptr, d.src_cell = _i(self._if["cells"]), _i(self._if["ptr"]), _i(self._if["src"])
            d.src_weight = _d(self._if["w"])
            descs = (IfaceDesc * 1)(d)
            nif = 1
            self.ni = d.n_faces
        h = C.c_void_p()
        _check(L.mrg_mesh_upload(ctx.h, self.n, self.nf, _i(self._lower), _i(self._upper), nif, descs,
                                 C.byref(h)))
        self.h = h
        ctx._meshes.append(self)

    def close(self):
        if self.h:
            _check(load().mrg_mesh_destroy(self.h))
            self.h = None

    def levels(self, ordering="exact") -> int:
        v = C.c_int()
        _check(load().mrg_mesh_levels(self.h, ORDERINGS[ordering], C.byref(v)))
        return v.value

    def set_blocks(self, bs, n_cells, lower, upper):
        """Declare this mesh the bs-expansion of the block mesh (n_cells,
        lower, upper), for the block preconditioner (precond="block")."""
        self._blo = np.ascontiguousarray(lower, dtype=np.int32)
        self._bup = np.ascontiguousarray(upper, dtype=np.int32)
        _check(load().mrg_mesh_set_blocks(self.h, int(bs), int(n_cells), len(self._blo), _i(self._blo),
                                          _i(self._bup)))

    def set_face_areas(self, sf):
        """The internal faces' area vectors ([n_faces, 3]) for GAMG's
        faceAreaPair agglomeration."""
        self._sf = np.ascontiguousarray(sf, dtype=np.float64).reshape(self.nf, 3)
        _check(load().mrg_mesh_set_face_areas(self.h, _d(self._sf)))

    def upload(self, diag, upper, lower=None, iface_bou=None, iface_int=None):
        self._c = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                   for a in (diag, upper, lower, iface_bou, iface_int)]
        _check(load().mrg_coeffs_upload(self.h, *[_d(a) for a in self._c]))

    def solve(self, b, x0, ctl: Controls | None = None, **kw):
        ctl = ctl if ctl is not None else controls(**kw)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        p = Perf()
        _check(load().mrg_solve(self.h, _d(b), _d(x), C.byref(ctl), C.byref(p)))
        return x, p.as_dict()

    def solve_device(self, d_b: int, d_x: int, ctl: Controls):
        p = Perf()
        _check(load().mrg_solve_device(self.h, C.c_void_p(d_b), C.c_void_p(d_x), C.byref(ctl), C.byref(p)))
        return p.as_dict()

    def amul(self, x, transpose=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        _check(load().mrg_amul(self.h, _d(x), _d(y), int(transpose)))
        return y

    def residual(self, b, x):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        r, nf = C.c_double(), C.c_double()
        _check(load().mrg_residual(self.h, _d(b), _d(x), C.byref(r), C.byref(nf)))
        return r.value, nf.value

    def precondition(self, precond, r, transpose=False, ordering="exact"):
        r = np.ascontiguousarray(r, dtype=np.float64)
        w = np.empty(self.n)
        _check(load().mrg_precondition(self.h, PRECONDITIONERS[precond], ORDERINGS[ordering], _d(r), _d(w),
                                       int(transpose)))
        return w

    def upload_device(self, d_diag, d_upper, d_lower=None, d_ibou=None, d_iint=None):
        vp = lambda p: None if p is None else C.c_void_p(p)
        _check(load().mrg_coeffs_upload_device(self.h, vp(d_diag), vp(d_upper), vp(d_lower), vp(d_ibou),
                                               vp(d_iint)))

    def tune(self, d_b: int, d_x: int, ctl: Controls) -> dict:
        """Autotune the launch shapes of this mesh's Krylov loop (device b, x)."""
        t = Tuning()
        _check(load().mrg_mesh_tune(self.h, C.c_void_p(d_b), C.c_void_p(d_x), C.byref(ctl), C.byref(t)))
        return t.as_dict()

    def time_kernel(self, ctl: Controls, kernel: int, reps: int) -> float:
        v = C.c_float()
        _check(load().mrg_time_kernel(self.h, C.byref(ctl), kernel, reps, C.byref(v)))
        return v.value

    def factor_diag(self, precond, ordering="exact"):
        out = np.empty(self.n)
        _check(load().mrg_factor_diag(self.h, PRECONDITIONERS[precond], ORDERINGS[ordering], _d(out)))
        return out


class Batch:
    """Independent systems solved in lockstep (each with its current coefficients)."""

    def __init__(self, ctx: Context, meshes, ordering="exact"):
        self.meshes = list(meshes)
        self.ordering = ordering
        arr = (C.c_void_p * len(self.meshes))(*[m.h.value for m in self.meshes])
        h = C.c_void_p()
        _check(load().mrg_batch_create(ctx.h, len(self.meshes), arr, ORDERINGS[ordering], C.byref(h)))
        self.h = h

    def solve(self, bs, x0s, ctl: Controls | None = None, **kw):
        kw.setdefault("ordering", self.ordering)
        ctl = ctl if ctl is not None else controls(**kw)
        ns = len(self.meshes)
        bs = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
        xs = [np.array(x, dtype=np.float64, copy=True) for x in x0s]
        pb = (C.POINTER(C.c_double) * ns)(*[_d(b) for b in bs])
        px = (C.POINTER(C.c_double) * ns)(*[_d(x) for x in xs])
        perfs = (Perf * ns)()
        _check(load().mrg_batch_solve(self.h, pb, px, C.byref(ctl), perfs))
        return xs, [p.as_dict() for p in perfs]

    def tune(self, d_bs, d_xs, ctl: Controls) -> dict:
        """Autotune the launch shapes of this batch's Krylov loop."""
        ns = len(self.meshes)
        t = Tuning()
        _check(load().mrg_batch_tune(self.h, (C.c_void_p * ns)(*d_bs), (C.c_void_p * ns)(*d_xs), C.byref(ctl),
                                     C.byref(t)))
        return t.as_dict()

    def solve_device(self, d_bs, d_xs, ctl: Controls):
        ns = len(self.meshes)
        pb = (C.c_void_p * ns)(*d_bs)
        px = (C.c_void_p * ns)(*d_xs)
        perfs = (Perf * ns)()
        _check(load().mrg_batch_solve_device(self.h, pb, px, C.byref(ctl), perfs))
        return [p.as_dict() for p in perfs]

    def close(self):
        if self.h:
            _check(load().mrg_batch_destroy(self.h))
            self.h = None


class Ggi:
    """Resident GGI weights: dst[i] = sum_k w_ik src[addr_ik]."""

    def __init__(self, ctx: Context, ptr, addr, w, n_src):
        self._ptr = np.ascontiguousarray(ptr, dtype=np.int32)
        self._addr = np.ascontiguousarray(addr, dtype=np.int32)
        self._w = np.ascontiguousarray(w, dtype=np.float64)
        self.n_dst = len(self._ptr) - 1
        self.n_src = int(n_src)
        h = C.c_void_p()
        _check(load().mrg_ggi_create(ctx.h, self.n_dst, self.n_src, _i(self._ptr), _i(self._addr), _d(self._w),
                                     C.byref(h)))
        self.h = h

    @classmethod
    def build(cls, ctx: Context, fa_ptr, fa_xy, fb_ptr, fb_xy, tol=1e-15):
        """Overlap weights of two planar patches built on the device
        (mrg_ggi_build).  Faces: CSR vertex pointers and (x, y) vertices,
        counter-clockwise.  Returns (a_from_b, b_from_a)."""
        pa = np.ascontiguousarray(fa_ptr, dtype=np.int32)
        xa = np.ascontiguousarray(fa_xy, dtype=np.float64)
        pb = np.ascontiguousarray(fb_ptr, dtype=np.int32)
        xb = np.ascontiguousarray(fb_xy, dtype=np.float64)
        ha, hb = C.c_void_p(), C.c_void_p()
        _check(load().mrg_ggi_build(ctx.h, len(pa) - 1, _i(pa), _d(xa), len(pb) - 1, _i(pb), _d(xb), float(tol),
                                    C.byref(ha), C.byref(hb)))
        out = []
        for h in (ha, hb):
            g = cls.__new__(cls)
            g.h = h
            nd, ns = C.c_int(), C.c_int()
            _check(load().mrg_ggi_get(h, C.byref(nd), C.byref(ns), None, None, None, None))
            g.n_dst, g.n_src = nd.value, ns.value
            out.append(g)
        return out[0], out[1]

    @classmethod
    def direct_map(cls, ctx: Context, centres_a, centres_b, tol):
        """Conformal face maps by face-centre match on the device
        (mrg_direct_map_build): one-weight GGIs (a_from_b, b_from_a)."""
        ca = np.ascontiguousarray(centres_a, dtype=np.float64).reshape(-1, 3)
        cb = np.ascontiguousarray(centres_b, dtype=np.float64).reshape(-1, 3)
        ha, hb = C.c_void_p(), C.c_void_p()
        _check(load().mrg_direct_map_build(ctx.h, len(ca), _d(ca), len(cb), _d(cb), float(tol), C.byref(ha),
                                           C.byref(hb)))
        out = []
        for h, nd, ns in ((ha, len(ca), len(cb)), (hb, len(cb), len(ca))):
            g = cls.__new__(cls)
            g.h = h
            g.n_dst, g.n_src = nd, ns
            out.append(g)
        return out[0], out[1]

    def csr(self):
        """The weights as (row_ptr, src_addr, w) host arrays."""
        nnz = C.c_int()
        _check(load().mrg_ggi_get(self.h, None, None, C.byref(nnz), None, None, None))
        ptr = np.empty(self.n_dst + 1, np.int32)
        addr = np.empty(max(nnz.value, 1), np.int32)
        w = np.empty(max(nnz.value, 1))
        _check(load().mrg_ggi_get(self.h, None, None, None, _i(ptr), _i(addr), _d(w)))
        return ptr, addr[:nnz.value], w[:nnz.value]

    def apply(self, src, ncomp=1):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.empty(self.n_dst * ncomp)
        _check(load().mrg_ggi_apply(self.h, _d(src), _d(dst), int(ncomp)))
        return dst if ncomp == 1 else dst.reshape(self.n_dst, ncomp)

    def apply_device(self, d_src: int, d_dst: int, ncomp=1):
        _check(load().mrg_ggi_apply_device(self.h, C.c_void_p(d_src), C.c_void_p(d_dst), int(ncomp)))

    def time_device(self, d_src: int, d_dst: int, reps: int, ncomp=1) -> float:
        """Mean ms per gather over `reps` back-to-back gathers (CUDA events)."""
        v = C.c_float()
        _check(load().mrg_ggi_time(self.h, C.c_void_p(d_src), C.c_void_p(d_dst), int(ncomp), int(reps),
                                   C.byref(v)))
        return float(v.value)

    def close(self):
        if self.h:
            _check(load().mrg_ggi_destroy(self.h))
            self.h = None


class Server:
    """Continuous-batching solve server (mrg_server_*).

    While it runs, use the context only through this object.  submit() keeps
    references to the request's arrays until the request is collected."""

    def __init__(self, ctx: Context, sym: Controls, asym: Controls | None = None, hbm_budget: int = 0,
                 max_active: int = 0):
        h = C.c_void_p()
        _check(load().mrg_server_create(ctx.h, C.byref(sym), C.byref(asym) if asym is not None else None,
                                        int(hbm_budget), int(max_active), C.byref(h)))
        self.h = h
        self._live = {}

    def submit(self, mesh: "Mesh", b, x0, diag, upper, lower=None, iface_bou=None, iface_int=None,
               asym: bool = False, x_out=None) -> int:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (diag, upper, lower, iface_bou, iface_int, b, x0)]
        x = np.empty(mesh.n) if x_out is None else x_out
        rid = C.c_uint64()
        _check(load().mrg_server_submit(self.h, mesh.h, int(bool(asym)),
                                        *[None if a is None else a.ctypes.data_as(C.c_void_p) for a in arrs],
                                        x.ctypes.data_as(C.c_void_p), C.byref(rid)))
        self._live[rid.value] = (arrs, x)
        return rid.value

    def _result(self, rid, fn, *extra):
        done = C.c_int()
        p = Perf()
        lat = C.c_double()
        rc = fn(self.h, C.c_uint64(rid), *extra, C.byref(done), C.byref(p), C.byref(lat))
        if done.value:
            _, x = self._live.pop(rid)
            _check(rc)
            return x, p.as_dict(), lat.value
        _check(rc)
        return None

    def poll(self, rid: int):
        """(x, perf, latency_ms) once the request finished, else None."""
        return self._result(rid, load().mrg_server_poll)

    def wait(self, rid: int, timeout_ms: float = -1.0):
        return self._result(rid, load().mrg_server_wait, C.c_double(timeout_ms))

    def stats(self) -> dict:
        s = ServerStats()
        _check(load().mrg_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_ if k != "reserved"}

    def close(self):
        if self.h:
            _check(load().mrg_server_destroy(self.h))
            self.h = None
            self._live.clear()


class DnInterface:
    """Device-resident partitioned Dirichlet-Neumann interface (mrg_dn_*).

    a / b: dicts with n_cells, face_cells, delta, k, area and the GGI CSR
    (ptr, addr, w) giving the patch's faces from the other patch's faces."""

    MODELS = {"fixed": 0, "aitken": 1, "IQNILS": 2}

    def __init__(self, ctx: Context, a: dict, b: dict, K=1.0, flux_jump=0.0, relax=0.75, model="aitken",
                 reuse=0, model_b=None, relax_b=None, reuse_b=None):
        """model / relax / reuse: the jump patch's accelerationModel (accType,
        relax, couplingReuse); the flux patch takes the same unless model_b /
        relax_b / reuse_b say otherwise."""
        self._keep = []

        def patch(p):
            arrs = [np.ascontiguousarray(p["face_cells"], np.int32), np.ascontiguousarray(p["delta"], np.float64),
                    np.ascontiguousarray(p["k"], np.float64), np.ascontiguousarray(p["area"], np.float64),
                    np.ascontiguousarray(p["ptr"], np.int32), np.ascontiguousarray(p["addr"], np.int32),
                    np.ascontiguousarray(p["w"], np.float64)]
            self._keep.append(arrs)
            return DnPatch(int(p["n_cells"]), len(arrs[0]), *[a_.ctypes.data_as(C.c_void_p) for a_ in arrs])

        cfg = DnConfig(float(K), float(flux_jump), float(relax), self.MODELS[model], int(reuse))
        h = C.c_void_p()
        _check(load().mrg_dn_create(ctx.h, C.byref(patch(a)), C.byref(patch(b)), C.byref(cfg), C.byref(h)))
        self.h = h
        if model_b is not None or relax_b is not None or reuse_b is not None:
            _check(load().mrg_dn_set_flux_relaxation(
                h, self.MODELS[model if model_b is None else model_b], float(relax if relax_b is None else relax_b),
                int(reuse if reuse_b is None else reuse_b)))
        self.na, self.nb = len(a["face_cells"]), len(b["face_cells"])

    def set_state(self, value_a, grad_b):
        _check(load().mrg_dn_set_state(self.h, _d(np.ascontiguousarray(value_a, np.float64)),
                                       _d(np.ascontiguousarray(grad_b, np.float64))))

    def new_time_step(self):
        _check(load().mrg_dn_new_time_step(self.h))

    def update_jump(self, d_t_b: int):
        _check(load().mrg_dn_update_jump(self.h, C.c_void_p(d_t_b)))

    def update_flux(self, d_t_a: int):
        _check(load().mrg_dn_update_flux(self.h, C.c_void_p(d_t_a)))

    def rhs(self, side: int, d_b0: int, d_b: int):
        _check(load().mrg_dn_rhs(self.h, int(side), C.c_void_p(d_b0), C.c_void_p(d_b)))

    def residuals(self, d_t_a: int, d_t_b: int):
        j, f = C.c_double(), C.c_double()
        _check(load().mrg_dn_residuals(self.h, C.c_void_p(d_t_a), C.c_void_p(d_t_b), C.byref(j), C.byref(f)))
        return j.value, f.value

    def state(self):
        va, gb, ai = np.empty(self.na), np.empty(self.nb), np.empty(2)
        _check(load().mrg_dn_get_state(self.h, _d(va), _d(gb), _d(ai)))
        return va, gb, ai

    def close(self):
        if self.h:
            _check(load().mrg_dn_destroy(self.h))
            self.h = None


class MonoInterface:
    """Monolithic interface coefficients of both sides of a regionCouple
    interface (mrg_mono_*).  a / b: dicts with n_cells, face_cells, w
    (patch weights), mld (magLongDelta), dc (deltaCoeffs), sf (|Sf|) and the
    GGI CSR (ptr, addr, wts) giving the patch's faces from the other
    side's faces.  Field arguments are device pointers."""

    def __init__(self, ctx: Context, a: dict, b: dict):
        self._keep = []

        def patch(p):
            arrs = [np.ascontiguousarray(p["face_cells"], np.int32)] + \
                   [np.ascontiguousarray(p[k], np.float64) for k in ("w", "mld", "dc", "sf")] + \
                   [np.ascontiguousarray(p["ptr"], np.int32), np.ascontiguousarray(p["addr"], np.int32),
                    np.ascontiguousarray(p["wts"], np.float64)]
            self._keep.append(arrs)
            return MonoPatch(int(p["n_cells"]), len(arrs[0]), *[a_.ctypes.data_as(C.c_void_p) for a_ in arrs])

        h = C.c_void_p()
        _check(load().mrg_mono_create(ctx.h, C.byref(patch(a)), C.byref(patch(b)), C.byref(h)))
        self.h = h

    def update(self, side, d_t_own, d_t_nbr, d_f_own, d_f_nbr, d_qr_own, d_qr_nbr, d_k, d_tw):
        p = lambda v: C.c_void_p(v) if v else None
        _check(load().mrg_mono_update(self.h, int(side), p(d_t_own), p(d_t_nbr), p(d_f_own), p(d_f_nbr),
                                      p(d_qr_own), p(d_qr_nbr), p(d_k), p(d_tw)))

    def source(self, side, d_t_own, d_t_nbr, d_tw, d_k, d_f_own, d_b):
        p = lambda v: C.c_void_p(v) if v else None
        _check(load().mrg_mono_source(self.h, int(side), p(d_t_own), p(d_t_nbr), p(d_tw), p(d_k), p(d_f_own),
                                      p(d_b)))

    def close(self):
        if self.h:
            _check(load().mrg_mono_destroy(self.h))
            self.h = None


def block_system(n: int, lower, upper, bs: int, diag, upper_c, lower_c=None):
    """A bs x bs block LDU system (foam-extend's BlockLduMatrix<vectorN> of
    fvBlockMatrix::solve, filesToReplace/fvBlockMatrix.C:1360-1388) as the
    scalar LDU system of bs n cells that Mesh takes (mrg_block_addressing /
    mrg_block_coeffs): diag [n, bs, bs], upper_c / lower_c [F, bs, bs]
    (lower_c None: the upper blocks transposed).  Returns (n_s, s_lower,
    s_upper, s_diag, s_upper_c, s_lower_c); cell c's component a is row
    bs c + a, so b and x are the block vectors flattened row-major."""
    L = load()
    lo = np.ascontiguousarray(lower, dtype=np.int32)
    up = np.ascontiguousarray(upper, dtype=np.int32)
    nf = len(lo)
    nfs = C.c_int()
    _check(L.mrg_block_addressing(n, nf, _i(lo), _i(up), bs, C.byref(nfs), None, None))   # checks bs first
    D = np.ascontiguousarray(diag, dtype=np.float64).reshape(n, bs, bs)
    U = np.ascontiguousarray(upper_c, dtype=np.float64).reshape(nf, bs, bs)
    Lc = None if lower_c is None else np.ascontiguousarray(lower_c, dtype=np.float64).reshape(nf, bs, bs)
    s_lower = np.empty(nfs.value, np.int32)
    s_upper = np.empty(nfs.value, np.int32)
    _check(L.mrg_block_addressing(n, nf, _i(lo), _i(up), bs, C.byref(nfs), _i(s_lower), _i(s_upper)))
    s_diag = np.empty(n * bs)
    s_uc = np.empty(nfs.value)
    s_lc = np.empty(nfs.value)
    _check(L.mrg_block_coeffs(n, nf, _i(lo), _i(up), bs, _d(D), _d(U), _d(Lc), _d(s_diag), _d(s_uc), _d(s_lc)))
    return n * bs, s_lower, s_upper, s_diag, s_uc, s_lc


def dn_criteria(corr, jump_res, flux_res, max_jump, max_flux) -> bool:
    return bool(load().mrg_dn_criteria(int(corr), float(jump_res), float(flux_res), float(max_jump),
                                       float(max_flux)))
