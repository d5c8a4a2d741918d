"""ctypes binding of the C ABI in include/skkr_gpu.h (libskkr_gpu.so).

There is no fallback: if the CUDA library is missing or no device is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libskkr_gpu.so")

SKKR_MAX_PRC = 16
NONREL, REL, BDG = 0, 1, 2
FP64, MIXED = 0, 1
ERRORS = {0: "ok", -1: "bad argument", -2: "CUDA error", -3: "decimation hit itermax",
          -4: "decimation diverged (error > 1e10)", -5: "unsupported input", -6: "out of device memory",
          -7: "non-finite result", -8: "another rank failed (or the reduction hook did)"}

I, D, P = C.c_int, C.c_double, C.c_void_p


class Sizes(C.Structure):
    _fields_ = [("mode", I), ("lmax", I), ("nprc", I), ("ninprc", I * (SKKR_MAX_PRC + 2)),
                ("bulkgeo", I), ("ngeff", I), ("itermaxl", I), ("itermaxr", I), ("errmax", D),
                ("itcpam", I), ("cpatol", D), ("precision", I), ("nk_chunk", I), ("slices", I)]


class RTable(C.Structure):
    _fields_ = [("nblk", I), ("nr", I), ("rstart", P), ("rvec", P), ("gR", P), ("nslot", I),
                ("mi", I), ("jmax", I), ("blkmap", P)]


class Status(C.Structure):
    _fields_ = [("code", I), ("ik", I), ("cpa_iterations", I), ("cpa_error", D),
                ("max_dec_iters", I), ("dec_iters_total", C.c_longlong),
                ("gpu_launches", C.c_longlong), ("max_refine_resid", D), ("run_ms", D),
                ("inv_fallbacks", C.c_longlong), ("k_fp64", C.c_longlong),
                ("inv_refined", C.c_longlong), ("alg_flops", D), ("graph_launches", C.c_longlong),
                ("graph_kernels", C.c_longlong)]


class KambeForm(C.Structure):
    _fields_ = [("e_re", D), ("e_im", D), ("nl", I), ("pos", P), ("alpha", P), ("centre", I), ("gvec", P),
                ("ng", I), ("rvec", P), ("nr", I), ("area", D), ("factor", D), ("gcut", D), ("rcut", D)]


class SkkrError(RuntimeError):
    def __init__(self, code, where=""):
        msg = "%s: %s (%d)" % (where, ERRORS.get(code, "error"), code)
        if code == -2:
            msg += ": " + last_error()
        super().__init__(msg)
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libskkr_gpu.so not built (run __graft_entry__.build()); "
                               "there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        L.skkr_gpu_create.argtypes = [P, P]
        L.skkr_gpu_destroy.argtypes = [P]
        L.skkr_gpu_stage.argtypes = [P, D, D, D, D, P, I, P, P, P, P, P, P, P, P, P, P, I]
        L.skkr_gpu_run.argtypes = [P, P]
        L.skkr_gpu_fetch.argtypes = [P, P, P, P, P, I]
        L.skkr_gpu_cpacoord.argtypes = [P, D, D, D, D, P, I, P, P, P, P, P, P, P, P, P, P, P, P, P, I, P]
        L.skkr_gpu_cpacoord_bdg.argtypes = [P, D, D, D, D, D, D, P, I, P, P, P, P, P, P, P, P, P, P, P, P, P,
                                            I, P]
        L.skkr_gpu_phystau.argtypes = [I, I, P, P, P, I]
        L.skkr_gpu_phystau2.argtypes = [I, I, P, P, P, P, P, I]
        L.skkr_gpu_mlp_forward.argtypes = [I, P, P, I, P, P]
        L.skkr_gpu_mlp_grad.argtypes = [I, P, P, I, P, P, P, P, P]
        L.skkr_gpu_mlp_train.argtypes = [I, P, P, I, P, P, P, I, D, D, I, P, P, P]
        L.skkr_gpu_kambe_dlm.argtypes = [I, D, D, P, P, I, P, I, P, I, D, D, D, D, P]
        L.skkr_gpu_kambe_alm.argtypes = [I, D, D, P, P, I, P, I, P, I, D, D, D, D, P]
        L.skkr_gpu_kambe_screened.argtypes = [I, D, D, P, I, P, P, I, P, I, P, I, D, D, D, D, I, I, P]
        L.skkr_gpu_layer_dos.argtypes = [I, I, I, P, I, P, P, I, P, P]
        L.skkr_gpu_bsf.argtypes = [I, I, I, I, P, P, P, P, P, P, P, P, I, P]
        L.skkr_gpu_tau2d.argtypes = [I, I, I, I, D, P, P, P, P, P, P]
        L.skkr_gpu_set_reduce.argtypes = [P, P, P]
        L.skkr_gpu_set_reduce_device.argtypes = [P, P, P]
        L.skkr_gpu_set_mixed_policy.argtypes = [P, D, D, I, D]
        L.skkr_gpu_set_graphs.argtypes = [P, I]
        L.skkr_gpu_set_newton.argtypes = [P, I]
        L.skkr_gpu_set_inverse_start.argtypes = [P, I]
        L.skkr_gpu_set_fused_split.argtypes = [P, I]
        L.skkr_gpu_stage_kambe.argtypes = [P, P]
        L.skkr_gpu_cpacoord_many.argtypes = [I, P, P, P]
        L.skkr_gpu_contour.argtypes = [P, I, P, P]
        L.skkr_gpu_gjinv_batch.argtypes = [I, I, P, I]
        L.skkr_gpu_surfgf_batch.argtypes = [I, I, P, P, P, P, I, I, D, P, P]
        L.skkr_gpu_gk.argtypes = [P, I, I, P, P]
        L.skkr_gpu_last_error.restype = C.c_char_p
        L.skkr_gpu_stage_slot.argtypes = [P, I, D, D, D, D, P, I, P, P, P, P, P, P, P, P, P, P, I]
        L.skkr_gpu_run_slot.argtypes = [P, I, P]
        L.skkr_gpu_fetch_slot.argtypes = [P, I, P, P, P, P, I]
        L.skkr_gpu_kernel_stats.argtypes = [I, P]
        L.skkr_gpu_tauij.argtypes = [P, I, P, P, P, P, P, P, P, I, P]
        _lib = L
    return _lib


def last_error() -> str:
    return lib().skkr_gpu_last_error().decode()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def cm(a):
    """(..., n, n) [row, col] -> column-major complex128 copy."""
    return np.array(np.swapaxes(np.asarray(a, np.complex128), -1, -2), order="C", copy=True)


def uncm(a):
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def _check(rc, where):
    if rc != 0:
        raise SkkrError(rc, where)


class EnergyArgs(C.Structure):
    _fields_ = [("ce_re", D), ("ce_im", D), ("fac_re", D), ("fac_im", D), ("fach_re", D), ("fach_im", D),
                ("rt", P), ("nk", I), ("xk", P), ("wk", P), ("lg", P), ("rg", P), ("conc", P),
                ("tminvl", P), ("tminvr", P), ("tminv", P), ("tminva", P), ("tminvb", P),
                ("tauc", P), ("taua", P), ("taub", P), ("ld", I)]


class RTableHolder:
    """Keeps the numpy buffers of an skkr_rtable alive."""

    def __init__(self, rt, blkmap, hole=None):
        self.rstart = np.ascontiguousarray(rt.rstart, np.int32)
        self.rvec = np.ascontiguousarray(rt.rvec, np.float64)
        # BdG: the hole table follows the electron table on the same R vectors
        self.gR = cm(rt.gR if hole is None else np.concatenate([rt.gR, hole.gR]))
        self.blkmap = np.ascontiguousarray(blkmap, np.int32)
        ns, mi, nj = self.blkmap.shape
        self.s = RTable(rt.nblk, len(self.rvec), _p(self.rstart), _p(self.rvec), _p(self.gR), ns, mi,
                        (nj - 1) // 2, _p(self.blkmap))

    def ptr(self):
        return C.cast(C.pointer(self.s), C.c_void_p)


def gjinv_batch(a):
    a = np.asarray(a, np.complex128)
    b, n, _ = a.shape
    buf = cm(a)
    _check(lib().skkr_gpu_gjinv_batch(n, b, _p(buf), n), "skkr_gpu_gjinv_batch")
    return uncm(buf)


def surfgf_batch(ml, m0, mr, itermax=50, errmax=1e-8):
    b, n, _ = m0.shape
    bl, b0, br = cm(ml), cm(m0), cm(mr)
    x = np.zeros_like(b0)
    it = np.zeros(b, np.int32)
    st = np.zeros(b, np.int32)
    _check(lib().skkr_gpu_surfgf_batch(n, b, _p(bl), _p(b0), _p(br), _p(x), n, itermax, errmax, _p(it),
                                       _p(st)), "skkr_gpu_surfgf_batch")
    return uncm(x), st, it


def gk(rt, blkmap, lmax, xk):
    h = RTableHolder(rt, blkmap)
    xk = np.ascontiguousarray(xk, np.float64)
    lm = (lmax + 1) ** 2
    out = np.zeros((len(xk), rt.nblk, lm, lm), np.complex128)
    _check(lib().skkr_gpu_gk(h.ptr(), lmax, len(xk), _p(xk), _p(out)), "skkr_gpu_gk")
    return uncm(out)


def phystau(tau, tinv, alpha, lmax, irel):
    t = cm(tau)
    ti = cm(tinv)
    al = np.ascontiguousarray(alpha, np.complex128)
    _check(lib().skkr_gpu_phystau(irel, lmax, _p(t), _p(ti), _p(al), t.shape[-1]), "skkr_gpu_phystau")
    return uncm(t)


def phystau2(tau, tinv1, alpha1, tinv2, alpha2, lmax, irel):
    """Pair block tau_ij screened -> physical on the device (skkr_gpu_phystau2):
    (1 + alpha1 tinv1) tau (1 + tinv2 alpha2), layer i's screening on the rows
    and layer j's on the columns."""
    t = cm(tau)
    t1 = cm(tinv1)
    t2 = cm(tinv2)
    a1 = np.ascontiguousarray(alpha1, np.complex128)
    a2 = np.ascontiguousarray(alpha2, np.complex128)
    _check(lib().skkr_gpu_phystau2(irel, lmax, _p(t), _p(t1), _p(a1), _p(t2), _p(a2), t.shape[-1]),
           "skkr_gpu_phystau2")
    return uncm(t)


def _mlp_args(layers):
    """dims (int32) and packed params (W_0, b_0, W_1, ...) of [(W, b), ...]."""
    dims = [layers[0][0].shape[0]] + [w.shape[1] for w, _ in layers]
    for (w, b), din, dout in zip(layers, dims[:-1], dims[1:]):
        if w.shape != (din, dout) or b.shape != (dout,):
            raise ValueError("layer shapes do not chain")
    params = np.concatenate([np.concatenate([np.ascontiguousarray(w, np.float64).ravel(),
                                             np.ascontiguousarray(b, np.float64)]) for w, b in layers])
    return np.array(dims, np.int32), params


def _mlp_unpack(dims, params):
    out, o = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        w = params[o:o + din * dout].reshape(din, dout).copy()
        o += din * dout
        out.append((w, params[o:o + dout].copy()))
        o += dout
    return out


def mlp_forward(layers, x):
    """Device forward of the warm-start MLP (skkr_gpu_mlp_forward)."""
    dims, params = _mlp_args(layers)
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros((len(x), dims[-1]))
    _check(lib().skkr_gpu_mlp_forward(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y)),
           "skkr_gpu_mlp_forward")
    return y


def mlp_grad(layers, x, y, rows=None):
    """Device loss and gradient [(dW, db), ...] (skkr_gpu_mlp_grad)."""
    dims, params = _mlp_args(layers)
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    r = None if rows is None else np.ascontiguousarray(rows, np.uint8)
    loss = np.zeros(1)
    grad = np.zeros_like(params)
    _check(lib().skkr_gpu_mlp_grad(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y),
                                   None if r is None else _p(r), _p(loss), _p(grad)), "skkr_gpu_mlp_grad")
    return float(loss[0]), _mlp_unpack(dims, grad)


def mlp_train(layers, x, y, rows, epochs, lr, weight_decay, eval_every=20):
    """Device full-batch AdamW training (skkr_gpu_mlp_train).  Returns
    (final layers, best layers, per-epoch training loss, (best held-out
    loss, training loss of that epoch))."""
    dims, params = _mlp_args(layers)
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    r = None if rows is None else np.ascontiguousarray(rows, np.uint8)
    tl = np.zeros(int(epochs))
    best = np.zeros(2)
    bp = np.zeros_like(params)
    _check(lib().skkr_gpu_mlp_train(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y),
                                    None if r is None else _p(r), int(epochs), float(lr), float(weight_decay),
                                    int(eval_every), _p(tl), _p(best), _p(bp)), "skkr_gpu_mlp_train")
    return _mlp_unpack(dims, params), _mlp_unpack(dims, bp), tl, (float(best[0]), float(best[1]))


def _mlp16_args(layers):
    dims, params = _mlp_args(layers)
    return dims, params.astype(np.float32)


def _mlp16_lib():
    L = lib()
    F = C.c_float
    L.skkr_gpu_mlp16_forward.argtypes = [I, P, P, I, P, P]
    L.skkr_gpu_mlp16_grad.argtypes = [I, P, P, I, P, P, P, P, P]
    L.skkr_gpu_mlp16_train.argtypes = [I, P, P, I, P, P, P, I, F, F, I, P, P, P]
    return L


class Mlp16Net:
    """A BF16-weight network kept on the device for repeated inference
    (skkr_gpu_mlp16_load / infer / free)."""

    def __init__(self, layers, maxrows=64):
        L = _mlp16_lib()
        L.skkr_gpu_mlp16_load.argtypes = [I, P, P, I, P]
        L.skkr_gpu_mlp16_infer.argtypes = [P, I, P, P]
        L.skkr_gpu_mlp16_free.argtypes = [P]
        self.dims, params = _mlp16_args(layers)
        self.maxrows = int(maxrows)
        h = C.c_void_p()
        _check(L.skkr_gpu_mlp16_load(len(layers), _p(self.dims), _p(params), self.maxrows,
                                     C.cast(C.pointer(h), C.c_void_p)), "skkr_gpu_mlp16_load")
        self.h = h
        self.L = L

    def __call__(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((len(x), self.dims[-1]), np.float32)
        _check(self.L.skkr_gpu_mlp16_infer(self.h, len(x), _p(x), _p(y)), "skkr_gpu_mlp16_infer")
        return y

    def close(self):
        if getattr(self, "h", None):
            self.L.skkr_gpu_mlp16_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp16_forward(layers, x):
    """Device forward of the BF16-weight network (skkr_gpu_mlp16_forward):
    FP32 master layers in, FP32 outputs."""
    dims, params = _mlp16_args(layers)
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros((len(x), dims[-1]), np.float32)
    _check(_mlp16_lib().skkr_gpu_mlp16_forward(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y)),
           "skkr_gpu_mlp16_forward")
    return y


def mlp16_grad(layers, x, y, rows=None):
    """Device loss and gradient [(dW, db), ...] of the BF16-weight network
    (skkr_gpu_mlp16_grad)."""
    dims, params = _mlp16_args(layers)
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    r = None if rows is None else np.ascontiguousarray(rows, np.uint8)
    loss = np.zeros(1, np.float32)
    grad = np.zeros_like(params)
    _check(_mlp16_lib().skkr_gpu_mlp16_grad(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y),
                                            None if r is None else _p(r), _p(loss), _p(grad)),
           "skkr_gpu_mlp16_grad")
    return float(loss[0]), _mlp_unpack(dims, grad)


def mlp16_train(layers, x, y, rows, epochs, lr, weight_decay, eval_every=20):
    """Device training of the BF16-weight network (skkr_gpu_mlp16_train);
    returns as mlp_train, FP32 master layers."""
    dims, params = _mlp16_args(layers)
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    r = None if rows is None else np.ascontiguousarray(rows, np.uint8)
    tl = np.zeros(int(epochs), np.float32)
    best = np.zeros(2, np.float32)
    bp = np.zeros_like(params)
    _check(_mlp16_lib().skkr_gpu_mlp16_train(len(layers), _p(dims), _p(params), len(x), _p(x), _p(y),
                                             None if r is None else _p(r), int(epochs), float(lr),
                                             float(weight_decay), int(eval_every), _p(tl), _p(best), _p(bp)),
           "skkr_gpu_mlp16_train")
    return _mlp_unpack(dims, params), _mlp_unpack(dims, bp), tl, (float(best[0]), float(best[1]))


def kambe_dlm(e, kxy, sep, lmax2, gvec, rvec, area, factor=1.0, gcut=12.0, rcut=40.0):
    """Device Kambe lattice sums D_L(k, s) of one energy for items (kxy[i],
    sep[i]) (skkr_gpu_kambe_dlm); returns (nitem, (lmax2+1)^2) complex."""
    kxy = np.ascontiguousarray(kxy, np.float64).reshape(-1, 2)
    sep = np.ascontiguousarray(sep, np.float64).reshape(-1, 3)
    g = np.ascontiguousarray(gvec, np.float64).reshape(-1, 2)
    r = np.ascontiguousarray(rvec, np.float64).reshape(-1, 2)
    out = np.zeros((len(kxy), 2 * (lmax2 + 1) ** 2))
    e = complex(e)
    _check(lib().skkr_gpu_kambe_dlm(len(kxy), e.real, e.imag, _p(kxy), _p(sep), lmax2, _p(g), len(g), _p(r), len(r),
                                    float(area), float(factor), float(gcut), float(rcut), _p(out)),
           "skkr_gpu_kambe_dlm")
    return out[:, 0::2] + 1j * out[:, 1::2]


def kambe_alm(e, kxy, sep, lmax, gvec, rvec, area, factor=1.0, gcut=12.0, rcut=40.0):
    """Device layer-pair structure constants alm(k, s) of one energy for items
    (kxy[i], sep[i]) (skkr_gpu_kambe_alm); returns (nitem, lmmax, lmmax)."""
    kxy = np.ascontiguousarray(kxy, np.float64).reshape(-1, 2)
    sep = np.ascontiguousarray(sep, np.float64).reshape(-1, 3)
    g = np.ascontiguousarray(gvec, np.float64).reshape(-1, 2)
    r = np.ascontiguousarray(rvec, np.float64).reshape(-1, 2)
    lm = (lmax + 1) ** 2
    out = np.zeros((len(kxy), 2 * lm * lm))
    e = complex(e)
    _check(lib().skkr_gpu_kambe_alm(len(kxy), e.real, e.imag, _p(kxy), _p(sep), lmax, _p(g), len(g), _p(r), len(r),
                                    float(area), float(factor), float(gcut), float(rcut), _p(out)),
           "skkr_gpu_kambe_alm")
    return (out[:, 0::2] + 1j * out[:, 1::2]).reshape(len(kxy), lm, lm)


def kambe_screened(e, kxy, pos, alpha, lmax, gvec, rvec, area, centre, jmax, factor=1.0, gcut=12.0, rcut=40.0):
    """Device screened G_scr(k) of the reference's slab form
    (skkr_gpu_kambe_screened); returns (nk, 2 jmax + 1, lmmax, lmmax)."""
    kxy = np.ascontiguousarray(kxy, np.float64).reshape(-1, 2)
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    al = np.ascontiguousarray(alpha, np.complex128).reshape(len(pos), lmax + 1)
    g = np.ascontiguousarray(gvec, np.float64).reshape(-1, 2)
    r = np.ascontiguousarray(rvec, np.float64).reshape(-1, 2)
    lm = (lmax + 1) ** 2
    out = np.zeros((len(kxy), 2 * jmax + 1, lm, lm), np.complex128)
    e = complex(e)
    _check(lib().skkr_gpu_kambe_screened(len(kxy), e.real, e.imag, _p(kxy), len(pos), _p(pos), _p(al), lmax, _p(g),
                                         len(g), _p(r), len(r), float(area), float(factor), float(gcut), float(rcut),
                                         int(centre), int(jmax), _p(out)), "skkr_gpu_kambe_screened")
    return out


REDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_longlong)


REDUCE_DEV_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p)


def reduce_device_callback(fn):
    """skkr_reduce_dev_fn around fn(ptr, n, stream): ptr the device address
    of n doubles, stream the library's cudaStream_t (as an int); an exception
    is reported to the library as a failed reduction."""
    def cb(_user, buf, n, stream):
        try:
            fn(int(buf), int(n), int(stream or 0))
            return 0
        except Exception:  # noqa: BLE001
            return 1
    return REDUCE_DEV_FN(cb)


def reduce_callback(fn):
    """skkr_reduce_fn around fn(buf: ndarray) that sums buf over the ranks in
    place; an exception is reported to the library as a failed reduction."""
    def cb(_user, buf, n):
        try:
            fn(np.ctypeslib.as_array(buf, shape=(int(n),)))
            return 0
        except Exception:  # noqa: BLE001
            return 1
    return REDUCE_FN(cb)


def layer_dos(tau, F, G, lmax, irel, para=False):
    """Layer DOS on the device from physical tau [nlay, nd, nd] and the radial
    integrals F, G [nlay, nd]: returns (zmom [nlay, nd], zdos_l [nlay, lmax+1]);
    the DOS is their imaginary part."""
    t = cm(np.asarray(tau, np.complex128).reshape((-1,) + np.shape(tau)[-2:]))
    nlay, nd = t.shape[0], t.shape[-1]
    f = np.ascontiguousarray(F, np.complex128).reshape(nlay, nd)
    g = np.ascontiguousarray(G, np.complex128).reshape(nlay, nd)
    zm = np.zeros((nlay, nd), np.complex128)
    zl = np.zeros((nlay, lmax + 1), np.complex128)
    _check(lib().skkr_gpu_layer_dos(irel, lmax, nlay, _p(t), nd, _p(f), _p(g), int(bool(para)), _p(zm), _p(zl)),
           "skkr_gpu_layer_dos")
    return zm, zl


def tau2d(m00, m01, m10, x, y, lk, wgeff=1.0):
    """tau2d on the device (skkr_gpu_tau2d): m00, m01, m10 [batch, nprc, n, n],
    x, y [batch, n, n], all [row, col]; returns wgeff times the layer-diagonal
    blocks [batch, nprc * n / lk, lk, lk]."""
    m00 = np.asarray(m00, np.complex128)
    batch, nprc, n = m00.shape[0], m00.shape[1], m00.shape[-1]
    args = [cm(m00), cm(m01), cm(m10), cm(x), cm(y)]
    out = np.zeros((batch, nprc * (n // lk), lk, lk), np.complex128)
    _check(lib().skkr_gpu_tau2d(batch, nprc, n, lk, float(wgeff), *[_p(a) for a in args], _p(out)), "skkr_gpu_tau2d")
    return uncm(out)


def bsf(mode, lmax, conc, tauk, tauc, taua, taub, F, Feh=None, pair=None, para=False):
    """Bloch spectral function on the device (skkr_gpu_bsf): tauk [nk, nlay,
    nd, nd] physical coherent tau of each k point, tauc / taua / taub [nlay,
    nd, nd] the k-integrated CPA taus, F [nlay, 2, 2, nd], for BdG Feh [nlay,
    2, 2, nde, nde] and pair [4, nde, nde] (singlet, T0, T-up, T-down), all
    [row, col].  Returns [nk, nlay, 6]: bsfe, bsfh, bsfeh, bsfhe, bsfteh,
    bsfthe (-1/pi Im of the sums)."""
    tk = np.asarray(tauk, np.complex128)
    nk, nlay, nd = tk.shape[0], tk.shape[1], tk.shape[-1]
    args = [cm(tk), cm(tauc), cm(taua), cm(taub)]
    f = np.ascontiguousarray(F, np.complex128).reshape(nlay, 2, 2, nd)
    fe = None if Feh is None else cm(np.asarray(Feh, np.complex128))
    pr = None if pair is None else cm(np.asarray(pair, np.complex128))
    out = np.zeros((nk, nlay, 6))
    c = np.ascontiguousarray(conc, np.float64)
    _check(lib().skkr_gpu_bsf(mode, lmax, nk, nlay, _p(c), *[_p(x) for x in args], _p(f),
                              None if fe is None else _p(fe), None if pr is None else _p(pr),
                              int(bool(para)), _p(out)), "skkr_gpu_bsf")
    return out


KSTAT_CLASSES = ("zgemm", "gjinv", "gk_ft", "other", "ozaki")


def kernel_stats_start():
    _check(lib().skkr_gpu_kernel_stats(1, None), "skkr_gpu_kernel_stats")


def kernel_stats_stop():
    out = np.zeros(4 * len(KSTAT_CLASSES))
    _check(lib().skkr_gpu_kernel_stats(0, _p(out)), "skkr_gpu_kernel_stats")
    return {name: dict(launches=int(out[4 * i]), ms=float(out[4 * i + 1]), work=float(out[4 * i + 2]),
                       work_fp64eq=float(out[4 * i + 3]))
            for i, name in enumerate(KSTAT_CLASSES)}


def zgemm_batch(a, b, precision="fp64", slices=5):
    a = np.asarray(a, np.complex128)
    nb, n, _ = a.shape
    A, B = cm(a), cm(b)
    Cm = np.zeros_like(A)
    L = lib()
    L.skkr_gpu_zgemm_batch.argtypes = [I, I, I, I, P, P, P, I]
    _check(L.skkr_gpu_zgemm_batch({"fp64": FP64, "mixed": MIXED}[precision], slices, n, nb, _p(A), _p(B),
                                  _p(Cm), n), "skkr_gpu_zgemm_batch")
    return uncm(Cm)


def autotune(force=None, report=False):
    """The Gauss-Jordan autotuner (skkr_gpu_autotune): force a layout (1..3),
    reset (0), and/or return the choices made so far."""
    L = lib()
    L.skkr_gpu_autotune.argtypes = [I, P, I]
    buf = C.create_string_buffer(512) if report else None
    _check(L.skkr_gpu_autotune(0 if force is None else int(force), buf, 512 if report else 0),
           "skkr_gpu_autotune")
    return buf.value.decode() if report else None


def zinv_batch(a, precision="fp64", newton=2):
    a = np.asarray(a, np.complex128)
    nb, n, _ = a.shape
    A = cm(a)
    r = np.zeros(1)
    L = lib()
    L.skkr_gpu_zinv_batch.argtypes = [I, I, I, P, I, I, P]
    _check(L.skkr_gpu_zinv_batch({"fp64": FP64, "mixed": MIXED}[precision], n, nb, _p(A), n, newton, _p(r)),
           "skkr_gpu_zinv_batch")
    return uncm(A), float(r[0])
