"""ctypes binding of ``lib/libctm_gb300.so`` (C ABI: ``include/ctm_gb300.h``).

There is no fallback: if the library is missing or CUDA is unavailable, the
first call raises.  Build the library with ``_build.build()`` (or
``__graft_entry__.build()``).
"""

import ctypes
import os

import torch

from . import _build

CTM_OK, CTM_ERR_INVALID, CTM_ERR_UNSUPPORTED, CTM_ERR_WORKSPACE = 0, 1, 2, 3
CTM_ERR_CUDA, CTM_ERR_NUMERIC, CTM_ERR_TIMEOUT = 4, 5, 6
PREC = {"fp64": 0, "mixed": 1, "bf16": 2}
PROJ = {"half-system": 0, "full-system": 1}
SVD = {"rsvd": 0, "full-rank": 1}

c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_vp = ctypes.c_void_p
c_sz_p = ctypes.POINTER(ctypes.c_size_t)


class CtmSite(ctypes.Structure):
    _fields_ = [("A", c_vp), ("C", c_vp * 4), ("E", c_vp * 4),
                ("c_rows", c_i64 * 4), ("c_cols", c_i64 * 4),
                ("e_rows", c_i64 * 4), ("e_cols", c_i64 * 4)]


class CtmOpts(ctypes.Structure):
    _fields_ = [("chi", c_i64), ("projectors", c_i32), ("svd_type", c_i32),
                ("svd_cutoff", ctypes.c_double), ("rsvd_niter", c_i32),
                ("rsvd_oversampling", c_i32), ("precision", c_i32), ("fixed_width", c_i32),
                ("mixed_floor", ctypes.c_double), ("mixed_flags", c_i32)]


SITE_P = ctypes.POINTER(CtmSite)
SITES_PP = ctypes.POINTER(SITE_P)

_SIGNATURES = {
    "ctm_version": ([], ctypes.c_char_p),
    "ctm_last_error": ([], ctypes.c_char_p),
    "ctm_device_status": ([ctypes.POINTER(ctypes.c_int), c_vp], ctypes.c_int),
    "ctm_set_mixed_contraction": ([c_i32, ctypes.POINTER(c_i32)], ctypes.c_int),
    "ctm_autotune": ([c_i32, ctypes.POINTER(c_i32)], ctypes.c_int),
    "ctm_autotune_entry": ([c_i32, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(c_i32),
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
                           ctypes.c_int),
    "ctm_kernel_launches": ([], ctypes.c_ulonglong),
    "ctm_qr_fallbacks": ([ctypes.POINTER(ctypes.c_ulonglong), c_vp], ctypes.c_int),
    "ctm_profile_begin": ([], None),
    "ctm_profile_end": ([], ctypes.c_int),
    "ctm_profile_query": ([ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)],
                          ctypes.c_int),
    "ctm_profile_kernel_count": ([ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "ctm_profile_kernel": ([ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)],
                           ctypes.c_int),
    "ctm_quarter_tensor": ([SITE_P, c_i64, c_i64, c_i32, c_vp, ctypes.POINTER(c_i64), c_i32,
                            c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_calculate_projectors": ([SITES_PP, c_i64, c_i64, c_i32, ctypes.POINTER(CtmOpts), c_vp,
                                  c_vp, c_vp, c_vp, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_projector_dims": ([SITES_PP, c_i64, c_i32, ctypes.POINTER(CtmOpts),
                            ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                            ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)], ctypes.c_int),
    "ctm_renormalize_boundary": ([SITE_P, c_i64, c_i64, c_i32, c_vp, c_i64, c_vp, c_i64, c_vp,
                                  c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_sz_p,
                                  c_vp], ctypes.c_int),
    "ctm_move_batched": ([SITE_P, c_i32, c_i32, c_i64, c_i64, ctypes.POINTER(c_i32), c_i32,
                          ctypes.POINTER(CtmOpts), ctypes.POINTER(c_vp), ctypes.POINTER(c_vp),
                          c_vp, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_site_rdm": ([SITE_P, c_i64, c_i64, c_i32, c_vp, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_bond_rdm": ([SITE_P, SITE_P, c_i64, c_i64, c_i32, c_i32, c_vp, c_vp, c_sz_p, c_vp],
                     ctypes.c_int),
    "ctm_norm_tensor": ([SITE_P, SITE_P, c_i64, c_i64, c_i32, c_vp, c_vp, c_i64, c_vp, c_vp,
                         c_sz_p, c_vp], ctypes.c_int),
    "ctm_als_solve": ([c_vp, c_vp, c_i64, c_i64, c_i64, c_i32, ctypes.c_double, c_i32,
                       ctypes.c_double, c_vp, c_vp, ctypes.POINTER(c_i32), c_vp,
                       ctypes.POINTER(ctypes.c_size_t), c_vp], ctypes.c_int),
    "ctm_als_cost": ([c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp,
                      ctypes.POINTER(ctypes.c_size_t), c_vp], ctypes.c_int),
    "ctm_svd_lowrank": ([c_vp, c_i64, c_i64, c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz_p,
                         c_vp], ctypes.c_int),
    "ctm_fused_matmul_svd_lowrank": ([c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i32, c_vp, c_vp,
                                      c_vp, c_vp, c_i32, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_fused_3matmul_svd_lowrank": ([c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64,
                                       c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz_p, c_vp],
                                      ctypes.c_int),
    "ctm_qr": ([c_vp, c_i64, c_i64, c_vp, c_i32, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_svd_f64": ([c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_svd_f32": ([c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_sz_p, c_vp], ctypes.c_int),
    "ctm_matmul": ([c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i32, c_vp, c_sz_p, c_vp],
                   ctypes.c_int),
    "ctm_matmul_mixed_noalloc": ([c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp], ctypes.c_int),
}

_lib = None


def library_path():
    return _build.LIB


def load():
    """Loads the library (once) and declares the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libctm_gb300.so not found at {path}; build it with "
                           "__graft_entry__.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(path)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGNATURES)


def check(status, what=""):
    if status == CTM_OK:
        return
    msg = load().ctm_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if status == CTM_ERR_INVALID:
        raise ValueError(text)
    raise RuntimeError(f"[ctm status {status}] {text}")


def require_cuda(t, name="tensor", storage=False):
    """CUDA float64 tensors; site tensors (``storage``) may also be stored in
    float32, which the library widens on entry (every contraction stays
    FP64 or mixed as configured) and the caller narrows on write-back."""
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the gb300 backend has no CPU path)")
    ok = (torch.float64, torch.float32) if storage else (torch.float64,)
    if t.dtype not in ok:
        raise ValueError(f"{name} must be float64{' or float32' if storage else ''}, got {t.dtype}")


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class _Workspace:
    """Scratch buffer per (device, stream), grown on demand and reused
    stream-ordered; calls on different streams never share one."""

    def __init__(self):
        self.buf = {}

    def get(self, nbytes, device):
        key = (torch.device(device).index, torch.cuda.current_stream(device).cuda_stream)
        b = self.buf.get(key)
        if b is None or b.numel() < nbytes:
            size = max(int(nbytes * 1.25), 1 << 20)
            b = torch.empty(size, dtype=torch.uint8, device=device)
            self.buf[key] = b
        return b


WORKSPACE = _Workspace()
_WS_CACHE = {}


def call(name, args_before_ws, device, key=None, stream=None):
    """Calls ``name(*args_before_ws, ws, &ws_bytes, stream)`` following the
    workspace protocol (size query, then the real call)."""
    lib = load()
    fn = getattr(lib, name)
    stream = stream_handle(device) if stream is None else stream
    # workspace sizes depend on the device (its SM count sets the split-K of
    # the tensor-core products), so the cache is keyed by device as well
    if key is not None:
        key = (torch.device(device).index, key)
    nbytes = _WS_CACHE.get(key) if key is not None else None
    if nbytes is None:
        sz = ctypes.c_size_t(0)
        check(fn(*args_before_ws, None, ctypes.byref(sz), stream), name)
        nbytes = sz.value
        if key is not None:
            _WS_CACHE[key] = nbytes
    ws = WORKSPACE.get(nbytes, device)
    sz = ctypes.c_size_t(ws.numel())
    check(fn(*args_before_ws, ctypes.c_void_p(ws.data_ptr()), ctypes.byref(sz), stream), name)


PROFILE_TAGS = {"gett_f64": 0, "tc_gemm": 1, "quarter": 2, "range_finder": 3, "orthonormalize": 4,
                "svd": 5, "projector_products": 6, "renormalize": 7, "gett_f32": 8,
                "tc_gemm_double_layer": 9}


def profile_begin():
    load().ctm_profile_begin()


def profile_end():
    """Returns {tag: (total_ms, total_work, launches)} of the profiled span."""
    lib = load()
    check(lib.ctm_profile_end(), "ctm_profile_end")
    out = {}
    for name, tag in PROFILE_TAGS.items():
        ms, work, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        check(lib.ctm_profile_query(tag, ctypes.byref(ms), ctypes.byref(work), ctypes.byref(n)),
              "ctm_profile_query")
        out[name] = (ms.value, work.value, n.value)
    return out


def profile_kernels():
    """Per-kernel table of the last profile (after ``profile_end``): a list
    of {name, unit ("flop" or "byte"), ms, work, launches}."""
    lib = load()
    n = ctypes.c_int(0)
    check(lib.ctm_profile_kernel_count(ctypes.byref(n)), "ctm_profile_kernel_count")
    out = []
    for i in range(n.value):
        name, unit = ctypes.c_char_p(), ctypes.c_int()
        ms, work, cnt = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        check(lib.ctm_profile_kernel(i, ctypes.byref(name), ctypes.byref(unit), ctypes.byref(ms),
                                     ctypes.byref(work), ctypes.byref(cnt)), "ctm_profile_kernel")
        out.append({"name": name.value.decode(), "unit": "byte" if unit.value else "flop",
                    "ms": ms.value, "work": work.value, "launches": cnt.value})
    return out


def qr_fallbacks(device=None):
    n = ctypes.c_ulonglong(0)
    check(load().ctm_qr_fallbacks(ctypes.byref(n), stream_handle(device)), "ctm_qr_fallbacks")
    return int(n.value)


CONTRACTION_FORMS = {"auto": 0, "double-layer": 1, "one-layer": 2}


def set_mixed_contraction(form):
    """Selects how the mixed path contracts the site tensors ("auto",
    "double-layer" or "one-layer"); returns the previous setting."""
    if form not in CONTRACTION_FORMS:
        raise ValueError(f"Invalid contraction form: {form} provided.")
    prev = c_i32(0)
    check(load().ctm_set_mixed_contraction(CONTRACTION_FORMS[form], ctypes.byref(prev)),
          "ctm_set_mixed_contraction")
    _WS_CACHE.clear()  # workspace sizes depend on the form
    return {v: k for k, v in CONTRACTION_FORMS.items()}[prev.value]


def autotune(enable=True, reset=False):
    """Turns the tile-plan autotuner of the tensor-core GEMMs on or off
    (``reset`` also forgets the tuned shapes); returns how many shapes are
    tuned.  Tuning happens on the first eager call of each product shape."""
    n = c_i32(0)
    if reset:
        check(load().ctm_autotune(-2, None), "ctm_autotune")
    check(load().ctm_autotune(1 if enable else 0, ctypes.byref(n)), "ctm_autotune")
    return n.value


def autotune_table():
    """The tuned shapes: dicts with M, N, K, passes, the chosen candidate
    (bit 0: 128-wide N tiles, bit 1: no K split) and both times in ms."""
    lib = load()
    n = c_i32(0)
    check(lib.ctm_autotune(-1, ctypes.byref(n)), "ctm_autotune")
    rows = []
    for i in range(n.value):
        mnk = (ctypes.c_int64 * 3)()
        mc = (c_i32 * 2)()
        best, dflt = ctypes.c_double(0), ctypes.c_double(0)
        check(lib.ctm_autotune_entry(i, mnk, mc, ctypes.byref(best), ctypes.byref(dflt)),
              "ctm_autotune_entry")
        rows.append({"M": mnk[0], "N": mnk[1], "K": mnk[2], "passes": mc[0], "choice": mc[1],
                     "best_ms": best.value, "default_ms": dflt.value})
    return rows


def kernel_launches():
    return int(load().ctm_kernel_launches())


def device_status(device=None):
    flags = ctypes.c_int(0)
    check(load().ctm_device_status(ctypes.byref(flags), stream_handle(device)), "ctm_device_status")
    return flags.value


class SiteRef:
    """A ``CtmSite`` over a site's A, C[0..3], E[0..3] tensors (kept alive)."""

    def __init__(self, site_tensor):
        A = site_tensor["A"]
        C = site_tensor["C"]
        E = site_tensor["E"]
        require_cuda(A, "A", storage=True)
        self.dtype = A.dtype  # storage type of the site (float64 or float32)
        self.keep = [A.to(torch.float64).contiguous()]
        self.D = A.shape[0]
        self.d = A.shape[4]
        s = CtmSite()
        s.A = self.keep[0].data_ptr()
        for k in range(4):
            ck = C[k]
            ek = E[k]
            require_cuda(ck, f"C[{k}]", storage=True)
            require_cuda(ek, f"E[{k}]", storage=True)
            ck = ck.to(torch.float64).contiguous()
            ek = ek.to(torch.float64).contiguous()
            self.keep += [ck, ek]
            s.C[k] = ck.data_ptr()
            s.E[k] = ek.data_ptr()
            s.c_rows[k], s.c_cols[k] = ck.shape
            s.e_rows[k], s.e_cols[k] = ek.shape[0], ek.shape[1]
        self.s = s
        self.device = A.device

    def shapes(self):
        s = self.s
        return tuple(tuple(x) for x in (s.c_rows, s.c_cols, s.e_rows, s.e_cols)) + (self.D, self.d)

    @property
    def pointer(self):
        return ctypes.pointer(self.s)


def opts_struct(config, chi, precision, fixed_width=False):
    o = CtmOpts()
    o.chi = int(chi)
    proj = getattr(config, "projectors", "half-system")
    proj = "full-system" if proj is None else proj
    if proj not in PROJ:
        raise ValueError(f"Invalid ctmrg projector type: {proj} provided.")
    svd = getattr(config, "svd_type", "rsvd")
    if svd not in SVD:
        raise ValueError(f"Invalid svd type: {svd} provided.")
    o.projectors = PROJ[proj]
    o.svd_type = SVD[svd]
    o.svd_cutoff = float(getattr(config, "svd_cutoff", 1e-12))
    o.rsvd_niter = int(getattr(config, "rsvd_niter", 2))
    o.rsvd_oversampling = int(getattr(config, "rsvd_oversampling", 2))
    if precision not in PREC:
        raise ValueError(f"Invalid precision: {precision} provided.")
    o.precision = PREC[precision]
    o.mixed_floor = float(getattr(config, "mixed_svd_floor", 1e-6))
    o.mixed_flags = int(getattr(config, "mixed_flags", 0))
    o.fixed_width = 1 if fixed_width else 0
    return o
