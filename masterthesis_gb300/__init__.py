"""GB300-native explicit-stencil engine for ScaFES problems.

This package holds the CUDA kernels and the C ABI (``csrc/``, built into
``libscafes_gb300.so``; declarations in ``include/scafes_gb300.h``) and a thin
ctypes binding used by the tests and the benchmark.  The C++ drop-in for
``ScaFES::Problem`` lives in ``masterthesis_gb300/scafes/``.

There is no CPU fallback: every call goes to the native library, and loading
fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libscafes_gb300.so"

# enum scafes_precision
PREC_F64, PREC_F32X2, PREC_F32, PREC_F64E = 0, 1, 2, 3
PRECISIONS = {"f64": PREC_F64, "f32x2": PREC_F32X2, "f32": PREC_F32, "f64e": PREC_F64E}
# enum scafes_field
(FIELD_U, FIELD_F_A, FIELD_F_B, FIELD_G_A, FIELD_G_B, FIELD_E_A, FIELD_E_B, FIELD_G_C, FIELD_G_D, FIELD_G_E,
 FIELD_C0, FIELD_CA) = range(12)
# enum scafes_border
BORDER_DIRICHLET, BORDER_MIRROR_POW2, BORDER_TABLE, BORDER_NODES = 0, 1, 2, 3
FLUX_NEUMANN, FLUX_CAUCHY, FLUX_RADIATION = 0, 1, 2

STATUS = {0: "SCAFES_OK", -1: "SCAFES_ERR_ARG", -2: "SCAFES_ERR_CUDA", -3: "SCAFES_ERR_STATE",
          -4: "SCAFES_ERR_UNSUPPORTED", -5: "SCAFES_ERR_NOMEM", -6: "SCAFES_ERR_TIMEOUT"}


class ScafesError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class BorderForm(C.Structure):
    """Mirror of ``struct scafes_border_form`` (one border class's rule)."""
    _fields_ = [("cu", C.c_double), ("cn", C.c_double * 6), ("cf", C.c_double), ("cg_old", C.c_double),
                ("cg_new", C.c_double), ("cu4", C.c_double)]


BorderForms = BorderForm * 64


class NodeRule(C.Structure):
    """Mirror of ``struct scafes_border_node_rule`` (one border node's rule)."""
    _fields_ = [("cu", C.c_double), ("cn", C.c_double * 6), ("cst", C.c_double)]


def node_rules_array(cu, cn, cst) -> np.ndarray:
    """The (m, 8) array of per-node border rules (cu, cn[0..5], cst) that
    set_border_node_rules takes, from arrays over the border nodes in
    Fortran order: cu (m,), cn (m, 6), cst (m,)."""
    m = len(cu)
    raw = np.empty((m, 8), dtype=np.float64)
    raw[:, 0] = cu
    raw[:, 1:7] = cn
    raw[:, 7] = cst
    return raw


class Cfg(C.Structure):
    """Mirror of ``struct scafes_cfg``."""
    _fields_ = [("dim", C.c_int), ("n_nodes", C.c_int * 3), ("coord_first", C.c_double * 3),
                ("coord_last", C.c_double * 3), ("tau", C.c_double), ("t_start", C.c_double),
                ("n_layers_at_border", C.c_int), ("precision", C.c_int), ("border", C.c_int),
                ("tile", C.c_int), ("c0", C.c_double), ("cp", C.c_double * 3), ("cf", C.c_double),
                ("stream", C.c_void_p)]


class BatchInstance(C.Structure):
    """Mirror of ``struct scafes_batch_instance``."""
    _fields_ = [("n_nodes", C.c_int * 3), ("coord_first", C.c_double * 3),
                ("coord_last", C.c_double * 3), ("tau", C.c_double), ("c0", C.c_double),
                ("cp", C.c_double * 3), ("cf", C.c_double), ("g_value", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with masterthesis_gb300.build.build_library() "
                "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.scafes_star7_heat_coeffs.argtypes = [C.POINTER(Cfg), C.c_double, C.c_double, C.c_double]
        L.scafes_gpu_create.argtypes = [C.POINTER(Cfg), C.POINTER(vp)]
        L.scafes_border_forms_flux.argtypes = [C.POINTER(Cfg), C.c_int, C.c_double, C.c_double,
                                               C.POINTER(BorderForm)]
        L.scafes_gpu_set_border_forms.argtypes = [vp, C.POINTER(BorderForm)]
        L.scafes_gpu_set_border_time_basis.argtypes = [vp, C.c_double, C.c_double]
        L.scafes_border_node_count.argtypes = [C.POINTER(Cfg), C.POINTER(C.c_longlong)]
        L.scafes_gpu_set_border_node_rules.argtypes = [vp, dp, C.c_size_t]
        L.scafes_gpu_step_snapshots.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_char_p]
        L.scafes_snapshot_info.argtypes = [C.c_char_p, C.c_int * 3, C.POINTER(C.c_int)]
        L.scafes_snapshot_read.argtypes = [C.c_char_p, C.c_int, dp, C.c_size_t, C.POINTER(C.c_longlong),
                                           C.POINTER(C.c_double)]
        L.scafes_gpu_upload.argtypes = [vp, C.c_int, dp, C.c_size_t]
        L.scafes_gpu_download.argtypes = [vp, C.c_int, dp, C.c_size_t]
        L.scafes_gpu_upload_async.argtypes = [vp, dp, C.c_size_t]
        L.scafes_gpu_download_async.argtypes = [vp, dp, C.c_size_t]
        L.scafes_gpu_synchronize.argtypes = [vp]
        L.scafes_gpu_step.argtypes = [vp, C.c_int]
        L.scafes_gpu_keep_initial.argtypes = [vp, C.c_int]
        L.scafes_gpu_adjoint.argtypes = [vp, dp, dp, dp, C.c_int]
        L.scafes_gpu_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.scafes_gpu_set_temporal_depth.argtypes = [vp, C.c_int]
        L.scafes_gpu_temporal_depth.argtypes = [vp, C.POINTER(C.c_int)]
        L.scafes_gpu_timestep.argtypes = [vp, C.POINTER(C.c_int)]
        L.scafes_gpu_err_linf.argtypes = [vp, dp, dp]
        L.scafes_gpu_last_step_ms.argtypes = [vp, C.POINTER(C.c_float)]
        L.scafes_gpu_last_step_launches.argtypes = [vp, C.POINTER(C.c_int)]
        L.scafes_gpu_last_error.argtypes = [vp]
        L.scafes_gpu_last_error.restype = C.c_char_p
        L.scafes_last_error.restype = C.c_char_p
        L.scafes_gpu_destroy.argtypes = [vp]
        L.scafes_gpu_destroy.restype = None
        bi = C.POINTER(BatchInstance)
        L.scafes_batch_star7_coeffs.argtypes = [bi, C.c_double, C.c_double, C.c_double]
        L.scafes_batch_create.argtypes = [bi, C.c_int, C.c_int, vp, C.POINTER(vp)]
        L.scafes_batch_upload.argtypes = [vp, C.c_int, C.c_int, dp, C.c_size_t]
        L.scafes_batch_download.argtypes = [vp, C.c_int, C.c_int, dp, C.c_size_t]
        L.scafes_batch_step.argtypes = [vp, C.c_int]
        L.scafes_batch_step_looped.argtypes = [vp, C.c_int]
        L.scafes_batch_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.scafes_batch_set_schedule.argtypes = [vp, C.c_int, C.c_int]
        L.scafes_batch_set_temporal_depth.argtypes = [vp, C.c_int]
        L.scafes_batch_temporal_depth.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_float),
                                                  C.POINTER(C.c_float)]
        L.scafes_batch_last_ms.argtypes = [vp, C.POINTER(C.c_float)]
        L.scafes_batch_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
        L.scafes_batch_last_error.argtypes = [vp]
        L.scafes_batch_last_error.restype = C.c_char_p
        L.scafes_batch_destroy.argtypes = [vp]
        L.scafes_batch_destroy.restype = None
        _lib = L
    return _lib


def _check(rc: int, h=None):
    if rc != 0:
        L = lib()
        msg = (L.scafes_gpu_last_error(h) if h else L.scafes_last_error()) or b""
        raise ScafesError(rc, msg.decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class HostArray:
    """A float64 numpy array in huge-page pinned host memory
    (scafes_host_alloc): the host side of uploads and downloads whose copies
    keep the link rate after long solves.  ``.a`` is the array; close()
    frees the memory (the array must not be used afterwards)."""

    def __init__(self, shape):
        L = lib()
        L.scafes_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
        L.scafes_host_free.argtypes = [C.c_void_p]
        L.scafes_host_free.restype = None
        n = int(np.prod(shape))
        self.p = C.c_void_p()
        _check(L.scafes_host_alloc(n * 8, C.byref(self.p)))
        self.a = np.ctypeslib.as_array((C.c_double * n).from_address(self.p.value)).reshape(shape)

    def close(self):
        if self.p:
            self.a = None
            lib().scafes_host_free(self.p)
            self.p = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def border_node_count(cfg: "Cfg") -> int:
    n = C.c_longlong()
    _check(lib().scafes_border_node_count(C.byref(cfg), C.byref(n)))
    return n.value


def make_cfg(n, first=(0.0, 0.0, 0.0), last=(1.0, 1.0, 1.0), tau=0.0, t_start=0.0,
             precision="f64", border=BORDER_DIRICHLET, c0=None, cp=None, cf=0.0,
             heat=None, stream=None, tile=0, n_layers=1) -> Cfg:
    """Builds a scafes_cfg.  ``heat=(coeff_a, rho_c, perf)`` fills the heat /
    Pennes coefficients via scafes_star7_heat_coeffs; otherwise give c0/cp/cf."""
    c = Cfg()
    c.dim = 3
    c.n_nodes[:] = list(n)
    c.coord_first[:] = list(first)
    c.coord_last[:] = list(last)
    c.tau, c.t_start = tau, t_start
    c.n_layers_at_border = n_layers
    c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    c.border = border
    c.tile = tile
    c.stream = stream
    if heat is not None:
        _check(lib().scafes_star7_heat_coeffs(C.byref(c), *heat))
    else:
        c.c0 = c0
        c.cp[:] = list(cp)
        c.cf = cf
    return c


SNAP_START, SNAP_END = 1, 2


def snapshot_info(path):
    """(n_nodes, count) of a snapshot file written by Plain.step_snapshots."""
    n, cnt = (C.c_int * 3)(), C.c_int()
    _check(lib().scafes_snapshot_info(str(path).encode(), n, C.byref(cnt)))
    return tuple(n), cnt.value


def snapshot_read(path, index):
    """(field (nz, ny, nx), step, time) of snapshot `index`."""
    n, _ = snapshot_info(path)
    a = np.empty((n[2], n[1], n[0]))
    st, tm = C.c_longlong(), C.c_double()
    _check(lib().scafes_snapshot_read(str(path).encode(), index, _dp(a), a.size, C.byref(st), C.byref(tm)))
    return a, st.value, tm.value


def border_forms_flux(cfg: Cfg, kind: int, lam: float = 1.0, alpha: float = 1.0):
    """The 64 border rules of the reference's Neumann / Cauchy / Radiation
    system tests for cfg (scafes_border_forms_flux)."""
    forms = BorderForms()
    _check(lib().scafes_border_forms_flux(C.byref(cfg), kind, lam, alpha, forms))
    return forms


class Plain:
    """One single-instance problem on the GPU (owns a scafes_handle)."""

    def __init__(self, cfg: Cfg):
        self.cfg = cfg
        self.n = tuple(cfg.n_nodes)
        h = C.c_void_p()
        _check(lib().scafes_gpu_create(C.byref(cfg), C.byref(h)))
        self.h = h

    @property
    def shape(self):
        return (self.n[2], self.n[1], self.n[0])

    def step_snapshots(self, n_steps: int, interval: int, path, flags: int = SNAP_START | SNAP_END):
        _check(lib().scafes_gpu_step_snapshots(self.h, n_steps, interval, flags, str(path).encode()), self.h)

    def set_temporal_depth(self, depth: int):
        _check(lib().scafes_gpu_set_temporal_depth(self.h, depth), self.h)

    @property
    def temporal_depth(self) -> int:
        d = C.c_int()
        _check(lib().scafes_gpu_temporal_depth(self.h, C.byref(d)), self.h)
        return d.value

    def set_border_forms(self, forms):
        _check(lib().scafes_gpu_set_border_forms(self.h, forms), self.h)

    def set_border_node_rules(self, rules: np.ndarray):
        """Per-node border rules (SCAFES_BORDER_NODES): an array (m, 8) of
        (cu, cn[0..5], cst) over the border nodes in Fortran order."""
        r = np.ascontiguousarray(rules, dtype=np.float64)
        if r.ndim != 2 or r.shape[1] != 8:
            raise ValueError("node rules must have shape (border nodes, 8)")
        _check(lib().scafes_gpu_set_border_node_rules(self.h, _dp(r), r.shape[0]), self.h)

    def set_border_time_basis(self, t_center: float, t_rate: float):
        """G(t) = sum_k G_k s^k with s = (time(t) - t_center) * t_rate."""
        _check(lib().scafes_gpu_set_border_time_basis(self.h, t_center, t_rate), self.h)

    def upload(self, field: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.size != int(np.prod(self.n)):
            raise ValueError(f"field has {a.size} values, grid has {int(np.prod(self.n))}")
        _check(lib().scafes_gpu_upload(self.h, field, _dp(a), a.size), self.h)

    def download(self, field: int = FIELD_U, out: np.ndarray | None = None) -> np.ndarray:
        a = np.empty(self.shape, dtype=np.float64) if out is None else out
        _check(lib().scafes_gpu_download(self.h, field, _dp(a), a.size), self.h)
        return a

    def step(self, n_steps: int):
        _check(lib().scafes_gpu_step(self.h, n_steps), self.h)

    def upload_async(self, arr: np.ndarray):
        """Enqueues the upload of the unknown field (scafes_gpu_upload_async):
        `arr` (C-contiguous float64, ideally page-locked, e.g. a HostArray)
        must stay unchanged until synchronize() returns."""
        if arr.dtype != np.float64 or not arr.flags.c_contiguous or arr.size != int(np.prod(self.n)):
            raise ValueError("upload_async needs a C-contiguous float64 array of the grid's size")
        _check(lib().scafes_gpu_upload_async(self.h, _dp(arr), arr.size), self.h)

    def download_async(self, out: np.ndarray):
        """Enqueues the download of the current iterate into `out`, valid once
        synchronize() returns."""
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != int(np.prod(self.n)):
            raise ValueError("download_async needs a C-contiguous float64 array of the grid's size")
        _check(lib().scafes_gpu_download_async(self.h, _dp(out), out.size), self.h)

    def synchronize(self):
        _check(lib().scafes_gpu_synchronize(self.h), self.h)

    def keep_initial(self, on: bool = True):
        """Keeps an FP64 device copy of every later upload of the unknown
        field: the state adjoint() starts from."""
        _check(lib().scafes_gpu_keep_initial(self.h, int(on)), self.h)

    def adjoint(self, dJ_du_T: np.ndarray, n_checkpoints: int = 45):
        """The backward entry: (dJ/dk, dJ/du0) of the steps run since the
        last upload, for the cotangent dJ/du_T (heat problems with a
        Dirichlet border constant in time; see scafes_gpu_adjoint)."""
        g = np.ascontiguousarray(dJ_du_T, dtype=np.float64)
        if g.size != int(np.prod(self.n)):
            raise ValueError(f"cotangent has {g.size} values, grid has {int(np.prod(self.n))}")
        gk, gu = np.empty(self.shape), np.empty(self.shape)
        _check(lib().scafes_gpu_adjoint(self.h, _dp(g), _dp(gk), _dp(gu), n_checkpoints), self.h)
        return gk, gu

    def autotune(self, n_steps: int = 20):
        """Picks the fastest sweep tile variant on this problem; returns
        (chosen 1-based variant, ms per step of each variant)."""
        chosen = C.c_int()
        ms = (C.c_float * 4)()
        _check(lib().scafes_gpu_autotune(self.h, n_steps, C.byref(chosen), ms), self.h)
        return chosen.value, list(ms)

    def timestep(self) -> int:
        t = C.c_int()
        _check(lib().scafes_gpu_timestep(self.h, C.byref(t)), self.h)
        return t.value

    def err_linf(self):
        e, m = C.c_double(), C.c_double()
        _check(lib().scafes_gpu_err_linf(self.h, C.byref(e), C.byref(m)), self.h)
        return e.value, m.value

    def last_step_ms(self) -> float:
        v = C.c_float()
        _check(lib().scafes_gpu_last_step_ms(self.h, C.byref(v)), self.h)
        return v.value

    def last_step_launches(self) -> int:
        v = C.c_int()
        _check(lib().scafes_gpu_last_step_launches(self.h, C.byref(v)), self.h)
        return v.value

    def close(self):
        if self.h:
            lib().scafes_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _bcheck(rc: int, b=None):
    if rc != 0:
        L = lib()
        msg = (L.scafes_batch_last_error(b) if b else L.scafes_last_error()) or b""
        raise ScafesError(rc, msg.decode())


def batch_instance(n, tau, coeff_a, rho_c=1.0, perf=0.0, g_value=0.0,
                   first=(0.0, 0.0, 0.0), last=(1.0, 1.0, 1.0)) -> BatchInstance:
    """One ensemble instance with star coefficients from the heat/Pennes
    parameters (scafes_batch_star7_coeffs)."""
    bi = BatchInstance()
    bi.n_nodes[:] = list(n)
    bi.coord_first[:] = list(first)
    bi.coord_last[:] = list(last)
    bi.tau = tau
    bi.g_value = g_value
    _bcheck(lib().scafes_batch_star7_coeffs(C.byref(bi), coeff_a, rho_c, perf))
    return bi


class BatchQueue:
    """An ensemble assembled one instance at a time (owns a
    scafes_gpu_batch: create / enqueue / run)."""

    def __init__(self, precision="f64", stream=None):
        L = lib()
        if not getattr(L, "_q_set", False):
            vp, dp = C.c_void_p, C.POINTER(C.c_double)
            L.scafes_gpu_batch_create.argtypes = [C.c_int, vp, C.POINTER(vp)]
            L.scafes_gpu_batch_enqueue.argtypes = [vp, C.POINTER(BatchInstance), dp, dp, C.POINTER(C.c_int)]
            L.scafes_gpu_batch_run.argtypes = [vp, C.c_int]
            L.scafes_gpu_batch_download.argtypes = [vp, C.c_int, dp, C.c_size_t]
            L.scafes_gpu_batch_ensemble.argtypes = [vp]
            L.scafes_gpu_batch_ensemble.restype = vp
            L.scafes_gpu_batch_last_error.argtypes = [vp]
            L.scafes_gpu_batch_last_error.restype = C.c_char_p
            L.scafes_gpu_batch_destroy.argtypes = [vp]
            L.scafes_gpu_batch_destroy.restype = None
            L._q_set = True
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = C.c_void_p()
        _check(L.scafes_gpu_batch_create(prec, stream, C.byref(h)))
        self.h = h
        self.shapes = []

    def _chk(self, rc):
        if rc != 0:
            raise ScafesError(rc, (lib().scafes_gpu_batch_last_error(self.h) or b"").decode())

    def enqueue(self, inst: BatchInstance, u0, f=None) -> int:
        a = np.ascontiguousarray(u0, dtype=np.float64)
        fa = None if f is None else np.ascontiguousarray(f, dtype=np.float64)
        idx = C.c_int()
        self._chk(lib().scafes_gpu_batch_enqueue(self.h, C.byref(inst), _dp(a), _dp(fa) if fa is not None else None,
                                                 C.byref(idx)))
        self.shapes.append((inst.n_nodes[2], inst.n_nodes[1], inst.n_nodes[0]))
        return idx.value

    def run(self, n_steps: int):
        self._chk(lib().scafes_gpu_batch_run(self.h, n_steps))

    def download(self, index: int) -> np.ndarray:
        a = np.empty(self.shapes[index], dtype=np.float64)
        self._chk(lib().scafes_gpu_batch_download(self.h, index, _dp(a), a.size))
        return a

    def close(self):
        if self.h:
            lib().scafes_gpu_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """An ensemble of independent instances advanced together (owns a
    scafes_batch)."""

    def __init__(self, instances, precision="f64", stream=None):
        arr = (BatchInstance * len(instances))(*instances)
        self.shapes = [(bi.n_nodes[2], bi.n_nodes[1], bi.n_nodes[0]) for bi in instances]
        h = C.c_void_p()
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        _bcheck(lib().scafes_batch_create(arr, len(instances), prec, stream, C.byref(h)))
        self.h = h

    def upload(self, inst: int, field: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _bcheck(lib().scafes_batch_upload(self.h, inst, field, _dp(a), a.size), self.h)

    def download(self, inst: int, field: int = FIELD_U) -> np.ndarray:
        a = np.empty(self.shapes[inst], dtype=np.float64)
        _bcheck(lib().scafes_batch_download(self.h, inst, field, _dp(a), a.size), self.h)
        return a

    def step(self, n_steps: int):
        _bcheck(lib().scafes_batch_step(self.h, n_steps), self.h)

    def step_looped(self, n_steps: int):
        _bcheck(lib().scafes_batch_step_looped(self.h, n_steps), self.h)

    def autotune(self, n_steps: int = 5):
        t, c = C.c_int(), C.c_int()
        _bcheck(lib().scafes_batch_autotune(self.h, n_steps, C.byref(t), C.byref(c)), self.h)
        return t.value, c.value

    def set_schedule(self, tile: int, ctas_per_sm: int = 0):
        _bcheck(lib().scafes_batch_set_schedule(self.h, tile, ctas_per_sm), self.h)

    def set_temporal_depth(self, depth: int):
        _bcheck(lib().scafes_batch_set_temporal_depth(self.h, depth), self.h)

    def temporal_depth(self) -> dict:
        """The depth in use and the autotuner's best ms per depth (-1 before
        an autotune)."""
        d, m1, m2 = C.c_int(), C.c_float(), C.c_float()
        _bcheck(lib().scafes_batch_temporal_depth(self.h, C.byref(d), C.byref(m1), C.byref(m2)), self.h)
        return {"depth": d.value, "ms_depth1": m1.value, "ms_depth2": m2.value}

    def last_ms(self) -> float:
        v = C.c_float()
        _bcheck(lib().scafes_batch_last_ms(self.h, C.byref(v)), self.h)
        return v.value

    def info(self) -> dict:
        it, la, ti, ct, nn = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        _bcheck(lib().scafes_batch_info(self.h, C.byref(it), C.byref(la), C.byref(ti), C.byref(ct),
                                        C.byref(nn)), self.h)
        return {"items": it.value, "launches": la.value, "tile": ti.value, "ctas_per_sm": ct.value,
                "nodes": nn.value}

    def close(self):
        if self.h:
            lib().scafes_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adjoint:
    """Gradient of J = 1/2 ||u_T - target||^2 for the flux-form
    variable-conductivity heat update (owns a scafes_adj)."""

    def __init__(self, n, tau, n_snapshots, first=(0.0, 0.0, 0.0), last=(1.0, 1.0, 1.0), stream=None,
                 precision="f64"):
        L = lib()
        if not getattr(L, "_adj_set", False):
            vp, dp = C.c_void_p, C.POINTER(C.c_double)
            i3, d3 = C.c_int * 3, C.c_double * 3
            L.scafes_adj_create.argtypes = [i3, d3, d3, C.c_double, C.c_int, vp, C.POINTER(vp)]
            L.scafes_adj_set_precision.argtypes = [vp, C.c_int]
            L.scafes_adj_set_conductivity.argtypes = [vp, dp, C.c_size_t]
            L.scafes_adj_set_conductivity_uniform.argtypes = [vp, C.c_double]
            L.scafes_adj_forward.argtypes = [vp, dp, C.c_int, dp, C.c_size_t]
            L.scafes_adj_gradient.argtypes = [vp, dp, dp, C.c_int, dp, dp, dp, C.c_size_t]
            L.scafes_adj_backward.argtypes = [vp, dp, dp, C.c_int, dp, dp, C.c_size_t]
            L.scafes_adj_stats.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]
            L.scafes_adj_schedule_cost.argtypes = [C.c_int, C.c_int]
            L.scafes_adj_schedule_cost.restype = C.c_longlong
            L.scafes_adj_last_error.argtypes = [vp]
            L.scafes_adj_last_error.restype = C.c_char_p
            L.scafes_adj_destroy.argtypes = [vp]
            L.scafes_adj_destroy.restype = None
            L._adj_set = True
        self.n = tuple(n)
        self.shape = (n[2], n[1], n[0])
        h = C.c_void_p()
        rc = L.scafes_adj_create((C.c_int * 3)(*n), (C.c_double * 3)(*first), (C.c_double * 3)(*last),
                                 tau, n_snapshots, stream, C.byref(h))
        if rc != 0:
            raise ScafesError(rc, (L.scafes_last_error() or b"").decode())
        self.h = h
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if prec != PREC_F64:
            self._chk(L.scafes_adj_set_precision(self.h, prec))

    def _chk(self, rc):
        if rc != 0:
            raise ScafesError(rc, (lib().scafes_adj_last_error(self.h) or b"").decode())

    def set_conductivity(self, k):
        a = np.ascontiguousarray(k, dtype=np.float64)
        self._chk(lib().scafes_adj_set_conductivity(self.h, _dp(a), a.size))

    def set_conductivity_uniform(self, k: float):
        self._chk(lib().scafes_adj_set_conductivity_uniform(self.h, float(k)))

    def forward(self, u0, n_steps):
        a = np.ascontiguousarray(u0, dtype=np.float64)
        out = np.empty(self.shape)
        self._chk(lib().scafes_adj_forward(self.h, _dp(a), n_steps, _dp(out), out.size))
        return out

    def gradient(self, u0, target, n_steps):
        a = np.ascontiguousarray(u0, dtype=np.float64)
        t = np.ascontiguousarray(target, dtype=np.float64)
        gk, gu = np.empty(self.shape), np.empty(self.shape)
        J = C.c_double()
        self._chk(lib().scafes_adj_gradient(self.h, _dp(a), _dp(t), n_steps, C.byref(J), _dp(gk), _dp(gu), gk.size))
        return J.value, gk, gu

    def backward(self, u0, dJ_duT, n_steps):
        """dJ/dk and dJ/du0 for a given cotangent dJ/du_T (scafes_adj_backward)."""
        a = np.ascontiguousarray(u0, dtype=np.float64)
        s = np.ascontiguousarray(dJ_duT, dtype=np.float64)
        gk, gu = np.empty(self.shape), np.empty(self.shape)
        self._chk(lib().scafes_adj_backward(self.h, _dp(a), _dp(s), n_steps, _dp(gk), _dp(gu), gk.size))
        return gk, gu

    def stats(self) -> dict:
        f, g = C.c_float(), C.c_float()
        fs, as_, s = C.c_longlong(), C.c_longlong(), C.c_int()
        self._chk(lib().scafes_adj_stats(self.h, C.byref(f), C.byref(g), C.byref(fs), C.byref(as_), C.byref(s)))
        return {"forward_ms": f.value, "gradient_ms": g.value, "forward_steps": fs.value,
                "adjoint_steps": as_.value, "snapshots": s.value}

    @staticmethod
    def schedule_cost(n_steps: int, n_snapshots: int) -> int:
        L = lib()
        L.scafes_adj_schedule_cost.argtypes = [C.c_int, C.c_int]
        L.scafes_adj_schedule_cost.restype = C.c_longlong
        return L.scafes_adj_schedule_cost(n_steps, n_snapshots)

    def close(self):
        if self.h:
            lib().scafes_adj_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Wide:
    """Fields with their own stencil width under the averaging update of the
    reference's StencilWidthVar test (owns a scafes_wide)."""

    def __init__(self, n, widths, stream=None):
        L = lib()
        if not getattr(L, "_wide_set", False):
            vp, dp = C.c_void_p, C.POINTER(C.c_double)
            L.scafes_wide_create.argtypes = [C.c_int * 3, C.c_int, C.POINTER(C.c_int), vp, C.POINTER(vp)]
            L.scafes_wide_upload.argtypes = [vp, C.c_int, dp, C.c_size_t]
            L.scafes_wide_download.argtypes = [vp, C.c_int, dp, C.c_size_t]
            L.scafes_wide_step.argtypes = [vp, C.c_int]
            L.scafes_wide_last_ms.argtypes = [vp, C.POINTER(C.c_float)]
            L.scafes_wide_last_error.argtypes = [vp]
            L.scafes_wide_last_error.restype = C.c_char_p
            L.scafes_wide_destroy.argtypes = [vp]
            L.scafes_wide_destroy.restype = None
            L._wide_set = True
        self.shape = (n[2], n[1], n[0])
        w = (C.c_int * len(widths))(*widths)
        h = C.c_void_p()
        rc = L.scafes_wide_create((C.c_int * 3)(*n), len(widths), w, stream, C.byref(h))
        if rc != 0:
            raise ScafesError(rc, (L.scafes_last_error() or b"").decode())
        self.h = h

    def _chk(self, rc):
        if rc != 0:
            raise ScafesError(rc, (lib().scafes_wide_last_error(self.h) or b"").decode())

    def upload(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(lib().scafes_wide_upload(self.h, field, _dp(a), a.size))

    def download(self, field):
        a = np.empty(self.shape)
        self._chk(lib().scafes_wide_download(self.h, field, _dp(a), a.size))
        return a

    def step(self, n_steps):
        self._chk(lib().scafes_wide_step(self.h, n_steps))

    def last_ms(self):
        v = C.c_float()
        self._chk(lib().scafes_wide_last_ms(self.h, C.byref(v)))
        return v.value

    def close(self):
        if self.h:
            lib().scafes_wide_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MF_LAME, MF_YEE = 0, 1


class MfCfg(C.Structure):
    """Mirror of ``struct scafes_mf_cfg``."""
    _fields_ = [("kind", C.c_int), ("n_nodes", C.c_int * 3), ("coord_first", C.c_double * 3),
                ("coord_last", C.c_double * 3), ("tau", C.c_double), ("t_start", C.c_double),
                ("precision", C.c_int), ("p", C.c_double * 8), ("src", C.c_int * 3), ("stream", C.c_void_p)]


class MultiField:
    """A multi-field leapfrog workload (Lame-Navier or Yee) on the GPU."""

    def __init__(self, kind, n, tau, params, precision="f64", src=(0, 0, 0), first=(0.0, 0.0, 0.0),
                 last=(1.0, 1.0, 1.0), t_start=0.0, stream=None):
        L = lib()
        if not getattr(L, "_mf_set", False):
            vp, dp = C.c_void_p, C.POINTER(C.c_double)
            L.scafes_mf_create.argtypes = [C.POINTER(MfCfg), C.POINTER(vp)]
            L.scafes_mf_upload.argtypes = [vp, C.c_int, dp, C.c_size_t]
            L.scafes_mf_download.argtypes = [vp, C.c_int, dp, C.c_size_t]
            L.scafes_mf_step.argtypes = [vp, C.c_int]
            L.scafes_mf_last_ms.argtypes = [vp, C.POINTER(C.c_float)]
            L.scafes_mf_last_error.argtypes = [vp]
            L.scafes_mf_last_error.restype = C.c_char_p
            L.scafes_mf_destroy.argtypes = [vp]
            L.scafes_mf_destroy.restype = None
            L._mf_set = True
        c = MfCfg()
        c.kind = kind
        c.n_nodes[:] = list(n)
        c.coord_first[:] = list(first)
        c.coord_last[:] = list(last)
        c.tau, c.t_start = tau, t_start
        c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        p = list(params) + [0.0] * (8 - len(params))
        c.p[:] = p
        c.src[:] = list(src)
        c.stream = stream
        self.shape = (n[2], n[1], n[0])
        h = C.c_void_p()
        rc = L.scafes_mf_create(C.byref(c), C.byref(h))
        if rc != 0:
            raise ScafesError(rc, (L.scafes_last_error() or b"").decode())
        self.h = h

    def _chk(self, rc):
        if rc != 0:
            raise ScafesError(rc, (lib().scafes_mf_last_error(self.h) or b"").decode())

    def upload(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(lib().scafes_mf_upload(self.h, field, _dp(a), a.size))

    def download(self, field):
        a = np.empty(self.shape)
        self._chk(lib().scafes_mf_download(self.h, field, _dp(a), a.size))
        return a

    def step(self, n_steps):
        self._chk(lib().scafes_mf_step(self.h, n_steps))

    def last_ms(self):
        v = C.c_float()
        self._chk(lib().scafes_mf_last_ms(self.h, C.byref(v)))
        return v.value

    def close(self):
        if self.h:
            lib().scafes_mf_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinTerm(C.Structure):
    """Mirror of ``struct scafes_lin_term``."""
    _fields_ = [("src", C.c_int), ("dx", C.c_int), ("dy", C.c_int), ("dz", C.c_int), ("w", C.c_double)]


LIN_MAX_FIELDS = 8
LIN_MAX_TERMS = 32


def _lin_bind(L):
    if getattr(L, "_lin_set", False):
        return
    vp, dp = C.c_void_p, C.POINTER(C.c_double)
    L.scafes_lin_create.argtypes = [C.c_int * 3, C.c_int, C.c_int, vp, C.POINTER(vp)]
    L.scafes_lin_set_rule.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(LinTerm), C.c_int, C.c_double]
    L.scafes_lin_upload.argtypes = [vp, C.c_int, dp, C.c_size_t]
    L.scafes_lin_download.argtypes = [vp, C.c_int, dp, C.c_size_t]
    L.scafes_lin_step.argtypes = [vp, C.c_int]
    L.scafes_lin_last_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.scafes_lin_last_error.argtypes = [vp]
    L.scafes_lin_last_error.restype = C.c_char_p
    L.scafes_lin_destroy.argtypes = [vp]
    L.scafes_lin_destroy.restype = None
    L._lin_set = True


class Linear:
    """Linear multi-field stencil rules with an optional leapfrog second
    phase (scafes_lin_*): the device form the drop-in Problem records from
    callbacks that couple several unknown fields.  Rules are set per
    (phase 1|2, field, node class 0..63); a term is (src, dx, dy, dz, w)."""

    def __init__(self, n, n_fields, n_phases=1, stream=None):
        L = lib()
        _lin_bind(L)
        self.shape = (n[2], n[1], n[0])
        h = C.c_void_p()
        rc = L.scafes_lin_create((C.c_int * 3)(*n), n_fields, n_phases, stream, C.byref(h))
        if rc != 0:
            raise ScafesError(rc, (L.scafes_last_error() or b"").decode())
        self.h = h

    def _chk(self, rc):
        if rc != 0:
            raise ScafesError(rc, (lib().scafes_lin_last_error(self.h) or b"").decode())

    def set_rule(self, phase, field, cls, terms, cst=0.0):
        arr = (LinTerm * max(1, len(terms)))(*[LinTerm(int(s), int(x), int(y), int(z), float(w))
                                               for s, x, y, z, w in terms])
        self._chk(lib().scafes_lin_set_rule(self.h, phase, field, cls, arr, len(terms), float(cst)))

    def upload(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(lib().scafes_lin_upload(self.h, field, _dp(a), a.size))

    def download(self, field):
        a = np.empty(self.shape)
        self._chk(lib().scafes_lin_download(self.h, field, _dp(a), a.size))
        return a

    def step(self, n_steps):
        self._chk(lib().scafes_lin_step(self.h, n_steps))

    def last_ms(self):
        v = C.c_float()
        self._chk(lib().scafes_lin_last_ms(self.h, C.byref(v)))
        return v.value

    def close(self):
        if self.h:
            lib().scafes_lin_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
