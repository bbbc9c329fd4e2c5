"""GB300 RNS-BFV hot path: a Python mirror of the fhe.rs API over libfheg.

The classes keep the names and argument meaning of the reference types
(fhe-math `rq::Context`, `rq::Poly`, `ntt::NttOperator`, `rq::Scaler`,
`rns::ScalingFactor`; fhe `bfv::BfvParameters`, `Ciphertext`,
`RelinearizationKey`, `EvaluationKey`/`GaloisKey`, `Multiplicator`) and call
the C ABI declared in include/fheg.h through ctypes. Device buffers are torch
tensors (int64 storage holding u64 residues bit for bit); torch is only used
for device memory and streams. Every compute call runs a CUDA kernel of
libfheg.so: there is no CPU fallback, and a missing library raises.
"""

from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfheg.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "fheg.h")

_lib = None

POWER_BASIS, NTT = 0, 1

c_u64 = ctypes.c_uint64
c_size = ctypes.c_size_t
P_u64 = ctypes.POINTER(ctypes.c_uint64)
c_vp = ctypes.c_void_p


class FhegError(RuntimeError):
    """A non-zero status returned by libfheg (see `fheg_status` in fheg.h)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


# Status codes (include/fheg.h `fheg_status`).
OK, ERR_INVALID_ARGUMENT, ERR_INVALID_MODULUS, ERR_NTT_UNSUPPORTED, ERR_INVALID_CONTEXT, ERR_INVALID_LEVEL, \
    ERR_KEY_MISMATCH, ERR_WRONG_PARTS, ERR_NO_MORE_CONTEXT, ERR_BUDGET, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED, \
    ERR_INTERNAL = range(14)


def build(force: bool = False) -> str:
    from importlib import util

    spec = util.spec_from_file_location("_fheg_build", os.path.join(_HERE, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib() -> ctypes.CDLL:
    """Loads libfheg.so. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with build() first (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


class _ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_size), ("streams", ctypes.c_uint32), ("max_batch", ctypes.c_uint32)]


class _Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int), ("par", c_vp), ("mult", c_vp), ("key", c_vp), ("exponent", c_size),
                ("level", c_size), ("in0", P_u64), ("in1", P_u64), ("out", P_u64)]


def _declare(L):
    i = ctypes.c_int
    sig = {
        "fheg_version": (ctypes.c_char_p, []),
        "fheg_status_string": (ctypes.c_char_p, [i]),
        "fheg_last_error": (ctypes.c_char_p, []),
        "fheg_kernel_launch_count": (c_u64, []),
        "fheg_multiply_groups": (i, [ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), ctypes.POINTER(c_vp),
                                     ctypes.POINTER(c_vp), ctypes.POINTER(c_size), c_size, c_vp]),
        "fheg_galois_relinearize_batch_capture": (i, [c_vp, ctypes.POINTER(c_vp), ctypes.POINTER(c_size),
                                                      ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), c_size,
                                                      ctypes.POINTER(c_vp)]),
        "fheg_ksk_to_bytes": (i, [c_vp, i, c_size, ctypes.c_char_p, c_size, ctypes.POINTER(c_size)]),
        "fheg_evaluation_key_to_bytes": (i, [ctypes.POINTER(c_vp), ctypes.POINTER(c_size), c_size, c_size, c_size,
                                             ctypes.c_char_p, c_size, ctypes.POINTER(c_size)]),
        "fheg_evaluation_key_from_bytes": (i, [c_vp, ctypes.c_char_p, c_size, ctypes.POINTER(c_vp),
                                               ctypes.POINTER(c_size), c_size, ctypes.POINTER(c_size),
                                               ctypes.POINTER(c_size), ctypes.POINTER(c_size)]),
        "fheg_poly_compute_shoup": (i, [c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_mul_shoup": (i, [c_vp, c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_ntt_cluster_set": (i, [ctypes.c_uint32, i]),
        "fheg_ntt_cluster_get": (i, [ctypes.c_uint32, ctypes.POINTER(i)]),
        "fheg_rns_tensor_set": (i, [i]),
        "fheg_rns_tensor_get": (i, [ctypes.POINTER(i)]),
        "fheg_rns_tensor_wait_failures": (i, [ctypes.POINTER(c_u64)]),
        "fheg_intpeak": (i, [i, c_size, ctypes.c_uint32, c_vp, c_vp, ctypes.POINTER(ctypes.c_double)]),
        "fheg_generate_prime": (i, [ctypes.c_uint32, c_u64, c_u64, P_u64]),
        "fheg_supports_ntt": (i, [c_u64, c_size]),
        "fheg_ntt_default_root": (i, [c_u64, c_size, P_u64]),
        "fheg_ntt_tables_host": (i, [c_u64, c_size, c_u64, P_u64, P_u64, P_u64, P_u64, P_u64]),
        "fheg_rns_scaler_constants_host": (i, [P_u64, c_size, P_u64, c_size, P_u64, c_size, P_u64, c_size, P_u64,
                                               c_size]),
        "fheg_context_create": (i, [P_u64, c_size, c_size, P_u64, ctypes.POINTER(c_vp)]),
        "fheg_context_destroy": (None, [c_vp]),
        "fheg_context_num_moduli": (c_size, [c_vp]),
        "fheg_context_degree": (c_size, [c_vp]),
        "fheg_ntt_forward": (i, [c_vp, c_vp, c_size, i, c_vp]),
        "fheg_ntt_backward": (i, [c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_op": (i, [c_vp, i, c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_substitute": (i, [c_vp, c_size, i, c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_switch_down": (i, [c_vp, i, c_vp, c_vp, c_size, c_vp]),
        "fheg_scaler_create": (i, [c_vp, c_vp, P_u64, c_size, P_u64, c_size, ctypes.POINTER(c_vp)]),
        "fheg_scaler_destroy": (None, [c_vp]),
        "fheg_scaler_scale": (i, [c_vp, i, c_vp, c_vp, c_size, c_vp]),
        "fheg_params_create": (i, [c_size, P_u64, c_size, c_u64, ctypes.POINTER(c_vp)]),
        "fheg_params_destroy": (None, [c_vp]),
        "fheg_params_context_at_level": (i, [c_vp, c_size, ctypes.POINTER(c_vp)]),
        "fheg_params_max_level": (c_size, [c_vp]),
        "fheg_ksk_create": (i, [c_vp, c_size, c_size, P_u64, P_u64, c_size, ctypes.POINTER(c_vp)]),
        "fheg_ksk_destroy": (None, [c_vp]),
        "fheg_ksk_create_seeded": (i, [c_vp, c_size, c_size, P_u64, ctypes.c_char_p, c_size, ctypes.POINTER(c_vp)]),
        "fheg_poly_random_from_seed": (i, [c_vp, c_vp, c_vp, c_size, c_size, c_vp]),
        "fheg_sample_cbd_from_seed": (i, [c_vp, c_size, c_size, c_size, c_vp, c_vp]),
        "fheg_ksk_from_bytes": (i, [c_vp, ctypes.c_char_p, c_size, i, ctypes.POINTER(c_vp), ctypes.POINTER(c_size),
                                    ctypes.POINTER(c_size), ctypes.POINTER(c_size)]),
        "fheg_ciphertext_serialized_size": (i, [c_vp, c_size, c_size, i, i, ctypes.POINTER(c_size)]),
        "fheg_ciphertext_to_bytes": (i, [c_vp, c_size, c_size, c_vp, c_size, ctypes.c_char_p, i, c_vp, c_size, c_vp]),
        "fheg_ciphertext_peek": (i, [c_vp, ctypes.c_char_p, c_size, ctypes.POINTER(c_size), ctypes.POINTER(c_size),
                                     ctypes.POINTER(i)]),
        "fheg_ciphertext_from_bytes": (i, [c_vp, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(c_size), c_size,
                                           c_size, c_size, c_vp, c_vp]),
        "fheg_relinearize": (i, [c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_galois_relinearize": (i, [c_vp, c_size, c_vp, c_vp, c_size, c_vp]),
        "fheg_rgsw_create": (i, [c_vp, c_size, P_u64, P_u64, P_u64, P_u64, ctypes.POINTER(c_vp)]),
        "fheg_rgsw_destroy": (None, [c_vp]),
        "fheg_external_product": (i, [c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_ciphertext_switch_down": (i, [c_vp, c_size, c_size, c_vp, c_vp, c_size, c_vp]),
        "fheg_ciphertext_add": (i, [c_vp, c_size, c_size, c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_multiplicator_create_default": (i, [c_vp, ctypes.POINTER(c_vp)]),
        "fheg_multiplicator_create": (i, [c_vp, c_size, P_u64, c_size, P_u64, c_size, P_u64, c_size, P_u64, c_size,
                                          P_u64, c_size, P_u64, c_size, P_u64, c_size, ctypes.POINTER(c_vp)]),
        "fheg_multiplicator_destroy": (None, [c_vp]),
        "fheg_multiplicator_enable_relinearization": (i, [c_vp, c_vp]),
        "fheg_multiplicator_enable_mod_switching": (i, [c_vp]),
        "fheg_multiplicator_output_shape": (i, [c_vp, ctypes.POINTER(c_size), ctypes.POINTER(c_size)]),
        "fheg_multiplicator_multiply": (i, [c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_multiplicator_multiply_host": (i, [c_vp, P_u64, P_u64, P_u64, c_size]),
        "fheg_multiplicator_set_host_pipeline": (i, [c_vp, c_size, i]),
        "fheg_relinearize_noalloc": (i, [c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_galois_relinearize_batch": (i, [c_vp, ctypes.POINTER(c_vp), ctypes.POINTER(c_size),
                                              ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), c_size, c_vp]),
        "fheg_poly_scalar_mul": (i, [c_vp, P_u64, c_size, c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_serialized_size": (i, [c_vp, ctypes.POINTER(c_size)]),
        "fheg_poly_serialize": (i, [c_vp, i, c_vp, c_vp, c_size, c_vp]),
        "fheg_poly_deserialize": (i, [c_vp, i, c_vp, c_vp, c_size, c_vp]),
        "fheg_dot_product_scalar": (i, [c_vp, c_size, c_size, c_vp, c_vp, c_size, c_size, c_vp, c_vp]),
        "fheg_inner_sum": (i, [c_vp, ctypes.POINTER(c_vp), ctypes.POINTER(c_size), c_size, c_vp, c_vp, c_size, c_vp]),
        "fheg_expand": (i, [c_vp, ctypes.POINTER(c_vp), ctypes.POINTER(c_size), c_size, c_size, c_vp, c_vp, c_vp]),
        "fheg_plaintext_encode": (i, [c_vp, c_size, c_vp, i, c_vp, c_size, c_vp]),
        "fheg_ciphertext_mul_plain": (i, [c_vp, c_size, c_size, c_vp, c_vp, i, c_vp, c_size, c_vp]),
        "fheg_secret_key_create": (i, [c_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(c_vp)]),
        "fheg_secret_key_destroy": (None, [c_vp]),
        "fheg_decrypt": (i, [c_vp, c_size, c_size, c_vp, i, c_vp, c_size, c_vp]),
        "fheg_encrypt": (i, [c_vp, c_size, c_vp, i, c_vp, c_vp, c_vp, c_size, c_vp]),
        "fheg_ciphertext_switch_to_level": (i, [c_vp, c_size, c_size, c_size, c_vp, c_vp, c_size, c_vp]),
        "fheg_device_alloc": (i, [c_size, ctypes.POINTER(c_vp)]),
        "fheg_device_free": (i, [c_vp]),
        "fheg_copy_to_device": (i, [c_vp, c_vp, c_size, c_vp]),
        "fheg_copy_to_host": (i, [c_vp, c_vp, c_size, c_vp]),
        "fheg_ntt_plan_set": (i, [ctypes.c_uint32, ctypes.c_uint32]),
        "fheg_ntt_prefetch_set": (i, [i]),
        "fheg_ntt_plan_get": (i, [ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_ntt_autotune": (i, [c_vp, c_size, c_vp, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_multiplicator_autotune": (i, [c_vp, c_size, c_vp, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_multiplicator_get_plan": (i, [c_vp, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_multiplicator_set_small_plan": (i, [c_vp, c_size, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_multiplicator_stage_times": (i, [c_vp, c_vp, c_vp, c_vp, c_size, c_vp, ctypes.POINTER(ctypes.c_float)]),
        "fheg_multiplicator_set_plan": (i, [c_vp, ctypes.POINTER(ctypes.c_uint32)]),
        "fheg_multiplicator_capture": (i, [c_vp, c_vp, c_vp, c_vp, c_size, ctypes.POINTER(c_vp)]),
        "fheg_graph_launch": (i, [c_vp, c_vp]),
        "fheg_graph_kernel_count": (i, [c_vp, ctypes.POINTER(c_u64)]),
        "fheg_graph_destroy": (None, [c_vp]),
        "fheg_server_create": (i, [ctypes.POINTER(_ServerConfig), ctypes.POINTER(c_vp)]),
        "fheg_server_destroy": (None, [c_vp]),
        "fheg_server_submit": (i, [c_vp, ctypes.POINTER(_Request), ctypes.POINTER(c_u64)]),
        "fheg_server_wait": (i, [c_vp, c_u64, ctypes.c_uint32]),
        "fheg_server_request_times": (i, [c_vp, c_u64, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
        "fheg_server_release": (i, [c_vp, c_u64]),
        "fheg_server_stats": (i, [c_vp, ctypes.POINTER(c_u64), ctypes.POINTER(c_u64), ctypes.POINTER(c_u64),
                                  ctypes.POINTER(c_size)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def check(status: int):
    if status != OK:
        raise FhegError(status, lib().fheg_last_error().decode())


def _u64(values) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(values, dtype=np.uint64))


def _ptr(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(P_u64)


def _words(x: int) -> np.ndarray:
    """Little-endian u64 words of a non-negative integer."""
    x = int(x)
    out = []
    while True:
        out.append(x & ((1 << 64) - 1))
        x >>= 64
        if x == 0:
            break
    return _u64(out)


def kernel_launch_count() -> int:
    return int(lib().fheg_kernel_launch_count())


INTPEAK_KINDS = {0: "mad.lo.u32", 1: "mad.wide.u32", 2: "mad.hi.u32", 3: "add.u32",
                 4: "NTT forward butterfly (64-bit Harvey, Shoup twiddle)",
                 5: "NTT inverse butterfly (64-bit Gentleman-Sande, Shoup twiddle)"}


def intpeak_launch(kind: int, blocks: int, iters: int, sink) -> float:
    """Launches one integer-throughput probe on the current stream (see
    fheg_intpeak) and returns the number of operations it performs."""
    ops = ctypes.c_double(0.0)
    check(lib().fheg_intpeak(kind, blocks, iters, _dp(sink), _stream(), ctypes.byref(ops)))
    return ops.value


# ---------------------------------------------------------------------------
# Device buffers (torch is plumbing only).


def _torch():
    import torch

    return torch


def to_device(arr: np.ndarray, device="cuda"):
    """Uploads a u64 numpy array to a device tensor (int64 storage)."""
    torch = _torch()
    a = np.ascontiguousarray(arr, dtype=np.uint64).view(np.int64)
    return torch.from_numpy(a.copy()).to(device)


def to_host(t) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint64)


def _dp(t) -> int:
    torch = _torch()
    assert t.is_cuda and t.dtype == torch.int64 and t.is_contiguous()
    return t.data_ptr()


def _stream() -> int:
    torch = _torch()
    return torch.cuda.current_stream().cuda_stream


def empty(shape, device="cuda"):
    torch = _torch()
    return torch.empty(tuple(shape), dtype=torch.int64, device=device)


# ---------------------------------------------------------------------------
# Host-only number theory (fhe-math zq / ntt).


def generate_prime(num_bits: int, modulo: int, upper_bound: int) -> Optional[int]:
    """fhe-math/src/zq/primes.rs:30-59 `generate_prime`."""
    out = c_u64(0)
    check(lib().fheg_generate_prime(num_bits, modulo, upper_bound, ctypes.byref(out)))
    return out.value or None


def supports_ntt(p: int, n: int) -> bool:
    return bool(lib().fheg_supports_ntt(p, n))


def ntt_default_root(p: int, n: int) -> int:
    out = c_u64(0)
    check(lib().fheg_ntt_default_root(p, n, ctypes.byref(out)))
    return out.value


def ntt_tables_host(p: int, n: int, root: int = 0):
    """The four twiddle tables and (size_inv, size_inv_shoup) of NttOperator::new."""
    t = [np.zeros(n, dtype=np.uint64) for _ in range(4)]
    inv = np.zeros(2, dtype=np.uint64)
    check(lib().fheg_ntt_tables_host(p, n, root, *[_ptr(x) for x in t], _ptr(inv)))
    return t, (int(inv[0]), int(inv[1]))


def rns_scaler_constants_host(from_moduli: Sequence[int], to_moduli: Sequence[int], num: int, den: int) -> dict:
    F, T = len(from_moduli), len(to_moduli)
    words = 5 + 2 * T + 2 * T * F + 5 * F
    out = np.zeros(words, dtype=np.uint64)
    fm, tm, nw, dw = _u64(from_moduli), _u64(to_moduli), _words(num), _words(den)
    check(lib().fheg_rns_scaler_constants_host(_ptr(fm), F, _ptr(tm), T, _ptr(nw), len(nw), _ptr(dw), len(dw),
                                               _ptr(out), words))
    o = 5
    r = {"theta_garner_shift": int(out[0]), "is_one": bool(out[1]),
         "theta_gamma": (int(out[2]), int(out[3]), bool(out[4]))}
    r["gamma"] = out[o:o + T]; o += T
    r["gamma_shoup"] = out[o:o + T]; o += T
    r["omega"] = out[o:o + T * F].reshape(T, F); o += T * F
    r["omega_shoup"] = out[o:o + T * F].reshape(T, F); o += T * F
    r["theta_omega_lo"] = out[o:o + F]; o += F
    r["theta_omega_hi"] = out[o:o + F]; o += F
    r["theta_omega_sign"] = out[o:o + F]; o += F
    r["theta_garner_lo"] = out[o:o + F]; o += F
    r["theta_garner_hi"] = out[o:o + F]; o += F
    return r


# ---------------------------------------------------------------------------
# fhe-math rq


class Context:
    """rq::Context (fhe-math/src/rq/context.rs:9-93), resident on the device."""

    def __init__(self, moduli: Sequence[int], degree: int, roots: Optional[Sequence[int]] = None, _handle=None,
                 _owner=None):
        self.moduli = [int(m) for m in moduli]
        self.degree = degree
        self._owner = _owner
        if _handle is not None:
            self._h = _handle
            self._owned = False
            return
        h = c_vp()
        m = _u64(self.moduli)
        r = _u64(roots) if roots is not None else None
        check(lib().fheg_context_create(_ptr(m), len(m), degree, _ptr(r) if r is not None else None,
                                        ctypes.byref(h)))
        self._h = h
        self._owned = True

    def __del__(self):
        if getattr(self, "_owned", False) and _lib is not None:
            _lib.fheg_context_destroy(self._h)
            self._owned = False

    @property
    def L(self) -> int:
        return len(self.moduli)

    def shape(self, count: int = 1):
        return (count, self.L, self.degree)


class NttOperator:
    """ntt::NttOperator (fhe-math/src/ntt/native.rs) for one modulus, applied
    to device buffers of shape [..., size]."""

    def __init__(self, p: int, size: int, root: Optional[int] = None):
        self.ctx = Context([p], size, [root] if root else None)
        self.size = size

    def forward(self, t, lazy: bool = False):
        """In place; `forward` (lazy=False) or `forward_vt_lazy` (lazy=True)."""
        check(lib().fheg_ntt_forward(self.ctx._h, _dp(t), t.numel() // self.size, int(lazy), _stream()))

    def backward(self, t):
        check(lib().fheg_ntt_backward(self.ctx._h, _dp(t), t.numel() // self.size, _stream()))


def ntt_forward(ctx: Context, t, lazy: bool = False):
    """Poly::into_ntt on a batch [count][L][N] (in place)."""
    count = t.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_ntt_forward(ctx._h, _dp(t), count, int(lazy), _stream()))


def ntt_backward(ctx: Context, t):
    """Poly::into_power_basis on a batch [count][L][N] (in place)."""
    count = t.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_ntt_backward(ctx._h, _dp(t), count, _stream()))


def ntt_plan_set(logn: int, block_logn: int):
    """Runs transforms of 2^logn as blocks of 2^block_logn (see fheg.h)."""
    check(lib().fheg_ntt_plan_set(logn, block_logn))


def ntt_prefetch_set(on: bool):
    """L2 prefetch of the next CTA's input rows in the NTT kernels (off by default)."""
    check(lib().fheg_ntt_prefetch_set(int(on)))


def ntt_cluster_set(logn: int, on: bool):
    """Single-pass cluster mode of the 2^12-block plan for 2^logn (see fheg.h)."""
    check(lib().fheg_ntt_cluster_set(logn, int(on)))


def ntt_cluster_get(logn: int) -> bool:
    out = ctypes.c_int(0)
    check(lib().fheg_ntt_cluster_get(logn, ctypes.byref(out)))
    return bool(out.value)


def rns_tensor_set(on: bool):
    """Tensor-core form of the exact RNS scalings (see fheg.h; on by default)."""
    check(lib().fheg_rns_tensor_set(int(on)))


def rns_tensor_get() -> bool:
    out = ctypes.c_int(0)
    check(lib().fheg_rns_tensor_get(ctypes.byref(out)))
    return bool(out.value)


def rns_tensor_wait_failures() -> int:
    """Bounded waits of the tensor-core scaler that ran out (0 when healthy)."""
    out = c_u64(0)
    check(lib().fheg_rns_tensor_wait_failures(ctypes.byref(out)))
    return out.value


def ntt_plan_get(logn: int) -> int:
    out = ctypes.c_uint32(0)
    check(lib().fheg_ntt_plan_get(logn, ctypes.byref(out)))
    return out.value


def ntt_autotune(ctx: Context, count: int = 64) -> int:
    """Times the valid plans for the context's degree and installs the fastest."""
    out = ctypes.c_uint32(0)
    check(lib().fheg_ntt_autotune(ctx._h, count, _stream(), ctypes.byref(out)))
    return out.value


def compute_shoup(ctx: Context, t):
    """Poly::compute_coefficients_shoup: the Shoup plane of Ntt values (the
    second half of an NttShoup polynomial)."""
    out = empty(t.shape, t.device)
    count = t.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_poly_compute_shoup(ctx._h, _dp(t), _dp(out), count, _stream()))
    return out


def mul_shoup(ctx: Context, a, b, b_shoup):
    """MulAssign<&Poly<NttShoup>> for Poly<Ntt>: a * b through b's Shoup plane."""
    out = empty(a.shape, a.device)
    count = a.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_poly_mul_shoup(ctx._h, _dp(a), _dp(b), _dp(b_shoup), _dp(out), count, _stream()))
    return out


def poly_op(ctx: Context, op: str, a, b=None):
    """Coefficient-wise `+`, `-`, `*` (Ntt x Ntt) or negation of batches."""
    code = {"add": 0, "sub": 1, "mul": 2, "neg": 3}[op]
    out = empty(a.shape, a.device)
    count = a.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_poly_op(ctx._h, code, _dp(a), _dp(b) if b is not None else None, _dp(out), count, _stream()))
    return out


def serialized_size(ctx: Context) -> int:
    out = c_size(0)
    check(lib().fheg_poly_serialized_size(ctx._h, ctypes.byref(out)))
    return out.value


def serialize(ctx: Context, t, representation: int):
    """Rq coefficient payloads (rq/convert.rs:17-42) of a batch [count][L][N]:
    a uint8 device tensor [count][bytes]."""
    torch = _torch()
    count = t.numel() // (ctx.L * ctx.degree)
    out = torch.empty((count, serialized_size(ctx)), dtype=torch.uint8, device=t.device)
    check(lib().fheg_poly_serialize(ctx._h, representation, _dp(t), out.data_ptr(), count, _stream()))
    return out


def deserialize(ctx: Context, payload, representation: int):
    """Inverse of serialize (rq/convert.rs:44-93): [count][bytes] -> [count][L][N]."""
    count = payload.shape[0]
    out = empty((count, ctx.L, ctx.degree), payload.device)
    check(lib().fheg_poly_deserialize(ctx._h, representation, payload.data_ptr(), _dp(out), count, _stream()))
    return out


def scalar_mul(ctx: Context, t, scalar: int):
    """MulAssign<&BigUint> for Poly (rq/ops.rs:297-352) on a batch [count][L][N]."""
    out = empty(t.shape, t.device)
    count = t.numel() // (ctx.L * ctx.degree)
    w = _words(scalar)
    check(lib().fheg_poly_scalar_mul(ctx._h, _ptr(w), len(w), _dp(t), _dp(out), count, _stream()))
    return out


def random_from_seed(ctx: Context, seeds, out=None, poly_stride: int = 0):
    """Poly::random_from_seed (rq/mod.rs:239-257) for a uint8 device tensor of
    seeds [count][32]: a new [count][L][N] tensor, or polynomial b written at
    out.data_ptr() + 8 * b * poly_stride (poly_stride in words; 2*L*N with
    out = ct[:, 1] fills the c1 of seeded ciphertexts [count][2][L][N])."""
    torch = _torch()
    if seeds.dtype != torch.uint8 or seeds.dim() != 2 or seeds.shape[1] != 32 or not seeds.is_cuda:
        raise FhegError(ERR_INVALID_ARGUMENT, "seeds must be a uint8 device tensor [count][32]")
    seeds = seeds.contiguous()
    count = seeds.shape[0]
    if out is None:
        out = empty((count, ctx.L, ctx.degree), seeds.device)
        ptr = _dp(out)
    else:
        assert out.is_cuda and out.dtype == torch.int64
        ptr = out.data_ptr()
    check(lib().fheg_poly_random_from_seed(ctx._h, seeds.data_ptr(), ptr, poly_stride, count, _stream()))
    return out


def sample_cbd_from_seed(seeds, variance: int, n: int):
    """sample_vec_cbd (fhe-util/src/lib.rs:22-55) of n samples per seed, from
    ChaCha8Rng::from_seed of each row of a uint8 device tensor [count][32]: a
    new int64 device tensor [count][n]."""
    torch = _torch()
    if seeds.dtype != torch.uint8 or seeds.dim() != 2 or seeds.shape[1] != 32 or not seeds.is_cuda:
        raise FhegError(ERR_INVALID_ARGUMENT, "seeds must be a uint8 device tensor [count][32]")
    seeds = seeds.contiguous()
    out = torch.empty((seeds.shape[0], n), dtype=torch.int64, device=seeds.device)
    check(lib().fheg_sample_cbd_from_seed(seeds.data_ptr(), variance, n, seeds.shape[0], out.data_ptr(),
                                          _stream()))
    return out


def ciphertext_serialized_size(par: BfvParameters, level: int, parts: int = 2, seeded: bool = False,
                               allow_variable_time: bool = False) -> int:
    out = c_size(0)
    check(lib().fheg_ciphertext_serialized_size(par._h, level, parts, int(seeded), int(allow_variable_time),
                                                ctypes.byref(out)))
    return out.value


def ciphertext_to_bytes(par: BfvParameters, level: int, ct, seeds: Optional[Sequence[bytes]] = None,
                        allow_variable_time: bool = False) -> List[bytes]:
    """Ciphertext::to_bytes (fhe/src/bfv/ciphertext.rs:164-191) of a batch
    [count][parts][L][N]; `seeds` (one 32-byte seed per ciphertext) replace
    the last parts."""
    count, parts = ct.shape[0], ct.shape[1]
    one = ciphertext_serialized_size(par, level, parts, seeds is not None, allow_variable_time)
    buf = ctypes.create_string_buffer(max(1, count * one))
    sd = b"".join(bytes(x) for x in seeds) if seeds is not None else None
    if sd is not None and len(sd) != 32 * count:
        raise FhegError(ERR_INVALID_ARGUMENT, "one 32-byte seed per ciphertext")
    check(lib().fheg_ciphertext_to_bytes(par._h, level, parts, _dp(ct), count, sd, int(allow_variable_time),
                                         ctypes.cast(buf, c_vp), count * one, _stream()))
    raw = buf.raw
    return [raw[b * one:(b + 1) * one] for b in range(count)]


def ciphertext_peek(par: BfvParameters, msg: bytes):
    """(level, parts, seeded) of a serialized Ciphertext."""
    level, parts, seeded = c_size(0), c_size(0), ctypes.c_int(0)
    check(lib().fheg_ciphertext_peek(par._h, bytes(msg), len(msg), ctypes.byref(level), ctypes.byref(parts),
                                     ctypes.byref(seeded)))
    return level.value, parts.value, bool(seeded.value)


def ciphertext_from_bytes(par: BfvParameters, msgs: Sequence[bytes], device="cuda"):
    """Ciphertext::from_bytes (ciphertext.rs:195-240) of messages of one
    level, part count and seededness: [count][parts][L][N] on the device."""
    level, parts, _ = ciphertext_peek(par, msgs[0])
    n = len(msgs)
    ctx = par.context_at_level(level)
    out = empty((n, parts, ctx.L, ctx.degree), device)
    arr = (ctypes.c_char_p * n)(*[bytes(m) for m in msgs])
    lens = (c_size * n)(*[len(m) for m in msgs])
    check(lib().fheg_ciphertext_from_bytes(par._h, arr, lens, n, level, parts, _dp(out), _stream()))
    return out


def substitute(ctx: Context, t, exponent: int, representation: int):
    """Poly::substitute (rq/mod.rs:319-369) on a batch."""
    out = empty(t.shape, t.device)
    count = t.numel() // (ctx.L * ctx.degree)
    check(lib().fheg_poly_substitute(ctx._h, exponent, representation, _dp(t), _dp(out), count, _stream()))
    return out


def switch_down(ctx: Context, t, representation: int):
    """Poly::switch_down (rq/mod.rs:390-448); returns [count][L-1][N]. `t` is
    consumed as scratch in Ntt representation."""
    count = t.numel() // (ctx.L * ctx.degree)
    out = empty((count, ctx.L - 1, ctx.degree), t.device)
    check(lib().fheg_poly_switch_down(ctx._h, representation, _dp(t), _dp(out), count, _stream()))
    return out


class ScalingFactor:
    """rns::ScalingFactor (fhe-math/src/rns/scaler.rs:19-47)."""

    def __init__(self, numerator: int, denominator: int):
        if denominator == 0:
            raise ValueError("denominator is zero")
        self.numerator, self.denominator = int(numerator), int(denominator)

    @staticmethod
    def one() -> "ScalingFactor":
        return ScalingFactor(1, 1)

    @property
    def is_one(self):
        return self.numerator == self.denominator


class Scaler:
    """rq::Scaler (fhe-math/src/rq/scaler.rs:17-126)."""

    def __init__(self, frm: Context, to: Context, factor: ScalingFactor):
        self.frm, self.to = frm, to
        n, d = _words(factor.numerator), _words(factor.denominator)
        h = c_vp()
        check(lib().fheg_scaler_create(frm._h, to._h, _ptr(n), len(n), _ptr(d), len(d), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_scaler_destroy(self._h)
            self._h = None

    def scale(self, t, representation: int):
        """Poly::scale on a batch [count][L_from][N] -> [count][L_to][N]."""
        count = t.numel() // (self.frm.L * self.frm.degree)
        out = empty((count, self.to.L, self.to.degree), t.device)
        check(lib().fheg_scaler_scale(self._h, representation, _dp(t), _dp(out), count, _stream()))
        return out


# ---------------------------------------------------------------------------
# fhe bfv


class BfvParameters:
    """bfv::BfvParameters (fhe/src/bfv/parameters.rs): the level chain."""

    def __init__(self, degree: int, moduli: Sequence[int], plaintext: int):
        self.degree, self.moduli, self.plaintext = degree, [int(m) for m in moduli], plaintext
        m = _u64(self.moduli)
        h = c_vp()
        check(lib().fheg_params_create(degree, _ptr(m), len(m), plaintext, ctypes.byref(h)))
        self._h = h
        self._ctx = {}

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_params_destroy(self._h)
            self._h = None

    def max_level(self) -> int:
        return len(self.moduli) - 1

    def context_at_level(self, level: int) -> Context:
        if level not in self._ctx:
            h = c_vp()
            check(lib().fheg_params_context_at_level(self._h, level, ctypes.byref(h)))
            self._ctx[level] = Context(self.moduli[:len(self.moduli) - level], self.degree, _handle=h, _owner=self)
        return self._ctx[level]


class KeySwitchingKey:
    """bfv KeySwitchingKey (fhe/src/bfv/keys/key_switching_key.rs:21-45),
    uploaded from its c0 / c1 polynomials ([count][L_ksk][N], Ntt values)."""

    def __init__(self, par: BfvParameters, c0: np.ndarray, c1: np.ndarray, ciphertext_level: int = 0,
                 ksk_level: int = 0):
        self.par = par
        self.ciphertext_level, self.ksk_level = ciphertext_level, ksk_level
        c0, c1 = _u64(c0), _u64(c1)
        h = c_vp()
        check(lib().fheg_ksk_create(par._h, ciphertext_level, ksk_level, _ptr(c0), _ptr(c1), c0.shape[0],
                                    ctypes.byref(h)))
        self._h = h

    KIND = 0  # message kind of fheg_ksk_from_bytes

    @classmethod
    def from_bytes(cls, par: BfvParameters, msg: bytes):
        """KeySwitchingKey / RelinearizationKey / GaloisKey::from_bytes
        (key_switching_key.rs:354-420): the key as the reference serialized it."""
        h, e, cl, kl = c_vp(), c_size(0), c_size(0), c_size(0)
        check(lib().fheg_ksk_from_bytes(par._h, bytes(msg), len(msg), cls.KIND, ctypes.byref(h), ctypes.byref(e),
                                        ctypes.byref(cl), ctypes.byref(kl)))
        k = cls.__new__(cls)
        k.par, k._h = par, h
        k.ciphertext_level, k.ksk_level = cl.value, kl.value
        if cls.KIND == 2:
            k.exponent = e.value
        return k

    def to_bytes(self) -> bytes:
        """KeySwitchingKey / RelinearizationKey / GaloisKey::to_bytes
        (key_switching_key.rs:332-352)."""
        n = c_size(0)
        e = getattr(self, "exponent", 0)
        check(lib().fheg_ksk_to_bytes(self._h, self.KIND, e, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        check(lib().fheg_ksk_to_bytes(self._h, self.KIND, e, buf, n.value, ctypes.byref(n)))
        return buf.raw[:n.value]

    @classmethod
    def from_seed(cls, par: BfvParameters, c0: np.ndarray, seed: bytes, ciphertext_level: int = 0,
                  ksk_level: int = 0, **kw):
        """A key from its c0 polynomials and the 32-byte seed of its c1
        (key_switching_key.rs:108-123, 383-406); c1 is expanded on the device."""
        if len(seed) != 32:
            raise FhegError(ERR_INVALID_ARGUMENT, "Invalid seed")
        k = cls.__new__(cls)
        k.par = par
        k.ciphertext_level, k.ksk_level = ciphertext_level, ksk_level
        for name, v in kw.items():
            setattr(k, name, v)
        c0 = _u64(c0)
        h = c_vp()
        check(lib().fheg_ksk_create_seeded(par._h, ciphertext_level, ksk_level, _ptr(c0), bytes(seed), c0.shape[0],
                                           ctypes.byref(h)))
        k._h = h
        return k

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_ksk_destroy(self._h)
            self._h = None


class RelinearizationKey(KeySwitchingKey):
    """bfv::RelinearizationKey (fhe/src/bfv/keys/relinearization_key.rs)."""

    KIND = 1

    def relinearizes(self, ct3):
        """relinearization_key.rs:71-98 on a batch [count][3][L][N]."""
        ctx = self.par.context_at_level(self.ciphertext_level)
        if ct3.dim() != 4 or ct3.shape[1] != 3:
            raise FhegError(ERR_WRONG_PARTS, "Only supports relinearization of ciphertext with 3 parts")
        count = ct3.shape[0]
        out = empty((count, 2, ctx.L, ctx.degree), ct3.device)
        check(lib().fheg_relinearize(self._h, _dp(ct3), _dp(out), count, _stream()))
        return out


class GaloisKey(KeySwitchingKey):
    """GaloisKey (fhe/src/bfv/keys/galois_key.rs) for one exponent."""

    KIND = 2

    def __init__(self, par, exponent: int, c0, c1, ciphertext_level: int = 0, ksk_level: int = 0):
        super().__init__(par, c0, c1, ciphertext_level, ksk_level)
        self.exponent = exponent % (2 * par.degree)

    @classmethod
    def from_seed(cls, par, exponent: int, c0, seed: bytes, ciphertext_level: int = 0, ksk_level: int = 0):
        """A Galois key from its c0 polynomials and the seed of its c1."""
        return super().from_seed(par, c0, seed, ciphertext_level, ksk_level, exponent=exponent % (2 * par.degree))

    def relinearize(self, ct):
        """galois_key.rs:63-124 on a batch [count][2][L][N]."""
        ctx = self.par.context_at_level(self.ciphertext_level)
        count = ct.shape[0]
        out = empty((count, 2, ctx.L, ctx.degree), ct.device)
        check(lib().fheg_galois_relinearize(self._h, self.exponent, _dp(ct), _dp(out), count, _stream()))
        return out


class RGSWCiphertext:
    """RGSWCiphertext (fhe/src/bfv/rgsw_ciphertext.rs:19-24) resident on the
    device, from its two key-switching keys' c0 / c1 polynomials ([L][L][N],
    Ntt values) at `level`."""

    def __init__(self, par: BfvParameters, ksk0_c0, ksk0_c1, ksk1_c0, ksk1_c1, level: int = 0):
        self.par, self.level = par, level
        arrs = [_u64(a) for a in (ksk0_c0, ksk0_c1, ksk1_c0, ksk1_c1)]
        ctx = par.context_at_level(level) if level <= par.max_level() else None
        if ctx is not None:
            for a in arrs:
                if a.shape != (ctx.L, ctx.L, par.degree):
                    raise FhegError(ERR_INVALID_ARGUMENT, f"key polynomials must be [{ctx.L}][{ctx.L}][{par.degree}]")
        h = c_vp()
        check(lib().fheg_rgsw_create(par._h, level, *[_ptr(a) for a in arrs], ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_rgsw_destroy(self._h)
            self._h = None

    def external_product(self, ct, out=None):
        """ct x RGSW (rgsw_ciphertext.rs:123-160) on a batch [count][2][L][N]."""
        ctx = self.par.context_at_level(self.level)
        if ct.dim() != 4 or ct.shape[1] != 2:
            raise FhegError(ERR_WRONG_PARTS, "Ciphertext must have two parts")
        if tuple(ct.shape[2:]) != (ctx.L, ctx.degree):
            raise FhegError(ERR_INVALID_LEVEL, "Ciphertext and RGSWCiphertext must have the same level")
        if out is None:
            out = empty(tuple(ct.shape), ct.device)
        check(lib().fheg_external_product(self._h, _dp(ct), _dp(out), ct.shape[0], _stream()))
        return out

    __mul__ = external_product  # Mul<&Ciphertext> for &RGSWCiphertext (rgsw_ciphertext.rs:155-160)


def evaluation_key_to_bytes(keys: Sequence["GaloisKey"], ciphertext_level: int, evaluation_key_level: int) -> bytes:
    """EvaluationKey::to_bytes (evaluation_key.rs:210-213, 382-392) of Galois keys."""
    k = len(keys)
    kh = (c_vp * k)(*[g._h for g in keys])
    ex = (c_size * k)(*[g.exponent for g in keys])
    n = c_size(0)
    check(lib().fheg_evaluation_key_to_bytes(kh, ex, k, ciphertext_level, evaluation_key_level, None, 0,
                                             ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value)
    check(lib().fheg_evaluation_key_to_bytes(kh, ex, k, ciphertext_level, evaluation_key_level, buf, n.value,
                                             ctypes.byref(n)))
    return buf.raw[:n.value]


def evaluation_key_from_bytes(par: BfvParameters, msg: bytes):
    """EvaluationKey::from_bytes (evaluation_key.rs:216-228, 394-432): its
    Galois keys, ciphertext level and evaluation key level."""
    msg = bytes(msg)
    count, cl, el = c_size(0), c_size(0), c_size(0)
    check(lib().fheg_evaluation_key_from_bytes(par._h, msg, len(msg), None, None, 0, ctypes.byref(count),
                                               ctypes.byref(cl), ctypes.byref(el)))
    hs = (c_vp * count.value)()
    ex = (c_size * count.value)()
    check(lib().fheg_evaluation_key_from_bytes(par._h, msg, len(msg), hs, ex, count.value, ctypes.byref(count),
                                               ctypes.byref(cl), ctypes.byref(el)))
    keys = []
    for h, e in zip(hs, ex):
        k = GaloisKey.__new__(GaloisKey)
        k.par, k._h, k.exponent = par, c_vp(h), int(e)
        k.ciphertext_level, k.ksk_level = cl.value, el.value
        keys.append(k)
    return keys, cl.value, el.value


class EvaluationKey:
    """EvaluationKey (fhe/src/bfv/keys/evaluation_key.rs:23-131): rotations."""

    def __init__(self, par: BfvParameters, galois_keys: Sequence[GaloisKey]):
        self.par = par
        self.gk = {g.exponent: g for g in galois_keys}

    def rotates_rows(self, ct):
        return self.gk[2 * self.par.degree - 1].relinearize(ct)

    def rotates_columns_by(self, ct, i: int):
        return self.gk[pow(3, i, 2 * self.par.degree)].relinearize(ct)


def rotate_batch(par: BfvParameters, keys: Sequence["GaloisKey"], cts: Sequence, outs: Sequence = None):
    """A ragged batch of GaloisKey::relinearize calls (one key, exponent and
    ciphertext per entry; ciphertexts may be at different levels), executed
    with one launch per stage."""
    n = len(keys)
    if outs is None:
        outs = [empty(c.shape, c.device) for c in cts]
    kh = (c_vp * n)(*[k._h for k in keys])
    ex = (c_size * n)(*[k.exponent for k in keys])
    ci = (c_vp * n)(*[_dp(c) for c in cts])
    co = (c_vp * n)(*[_dp(o) for o in outs])
    check(lib().fheg_galois_relinearize_batch(par._h, kh, ex, ci, co, n, _stream()))
    return outs


def capture_rotate_batch(par: BfvParameters, keys: Sequence["GaloisKey"], cts: Sequence, outs: Sequence):
    """The ragged batch of rotate_batch recorded once as a CUDA graph over
    fixed buffers; launch() replays it."""
    n = len(keys)
    kh = (c_vp * n)(*[k._h for k in keys])
    ex = (c_size * n)(*[k.exponent for k in keys])
    ci = (c_vp * n)(*[_dp(c) for c in cts])
    co = (c_vp * n)(*[_dp(o) for o in outs])
    h = c_vp()
    check(lib().fheg_galois_relinearize_batch_capture(par._h, kh, ex, ci, co, n, ctypes.byref(h)))
    return MultiplyGraph(h, (par, list(keys), list(cts), list(outs)))


def ciphertext_switch_down(par: BfvParameters, level: int, ct):
    """Ciphertext::switch_down (fhe/src/bfv/ciphertext.rs:86-97) on a batch
    [count][parts][L][N]; `ct` is consumed as scratch."""
    count, parts = ct.shape[0], ct.shape[1]
    ctx = par.context_at_level(level)
    out = empty((count, parts, ctx.L - 1, ctx.degree), ct.device)
    check(lib().fheg_ciphertext_switch_down(par._h, level, parts, _dp(ct), _dp(out), count, _stream()))
    return out


def ciphertext_switch_to_level(par: BfvParameters, level: int, target_level: int, ct):
    """Ciphertext::switch_to_level (fhe/src/bfv/ciphertext.rs:100-119) on a
    batch [count][parts][L][N]; `ct` is consumed as scratch."""
    count, parts = ct.shape[0], ct.shape[1]
    ctx = par.context_at_level(target_level) if target_level <= len(par.moduli) - 1 else None
    out = empty((count, parts, ctx.L if ctx else 1, par.degree), ct.device)
    check(lib().fheg_ciphertext_switch_to_level(par._h, level, target_level, parts, _dp(ct), _dp(out), count,
                                                _stream()))
    return out


def plaintext_encode(par: BfvParameters, level: int, values, simd: bool = True):
    """Plaintext::poly_ntt of each row of `values` [count][N] (< t), device in
    and out (plaintext_vec.rs:40-100)."""
    count = values.shape[0]
    ctx = par.context_at_level(level)
    out = empty((count, ctx.L, par.degree), values.device)
    check(lib().fheg_plaintext_encode(par._h, level, _dp(values), int(simd), _dp(out), count, _stream()))
    return out


def ciphertext_mul_plain(par: BfvParameters, level: int, ct, pt_ntt):
    """MulAssign<&Plaintext> for Ciphertext (ops/mod.rs:229-238) on a batch
    [count][parts][L][N]; pt_ntt is [L][N] (shared) or [count][L][N]."""
    out = empty(ct.shape, ct.device)
    per_ct = int(pt_ntt.dim() == 3)
    check(lib().fheg_ciphertext_mul_plain(par._h, level, ct.shape[1], _dp(ct), _dp(pt_ntt), per_ct, _dp(out),
                                          ct.shape[0], _stream()))
    return out


def dot_product_scalar(par: BfvParameters, level: int, cts, pts):
    """ops/dot_product.rs:56-140: sum_c cts[g][c] * pts[c] for every group g.
    cts [groups][count][parts][L][N] (or [count][parts][L][N] for one group),
    pts [count][L][N] (plaintext Ntt polynomials)."""
    single = cts.dim() == 4
    if single:
        cts = cts[None]
    groups, count, parts = cts.shape[0], cts.shape[1], cts.shape[2]
    out = empty((groups, parts, cts.shape[3], cts.shape[4]), cts.device)
    check(lib().fheg_dot_product_scalar(par._h, level, parts, _dp(cts.contiguous()), _dp(pts), count, groups,
                                        _dp(out), _stream()))
    return out[0] if single else out


def _keys(keys):
    n = len(keys)
    return (c_vp * n)(*[k._h for k in keys]), (c_size * n)(*[k.exponent for k in keys]), n


def inner_sum(par: BfvParameters, keys: Sequence["GaloisKey"], ct):
    """EvaluationKey::computes_inner_sum (evaluation_key.rs:56-83) on a batch
    [count][2][L][N]; keys in the order of ora.EvaluationKey.inner_sum_exponents."""
    kh, ex, n = _keys(keys)
    out = empty(ct.shape, ct.device)
    check(lib().fheg_inner_sum(par._h, kh, ex, n, _dp(ct), _dp(out), ct.shape[0], _stream()))
    return out


def expand(par: BfvParameters, keys: Sequence["GaloisKey"], ct, size: int):
    """EvaluationKey::expands (evaluation_key.rs:148-193): [2][L][N] -> [size][2][L][N]."""
    kh, ex, n = _keys(keys)
    out = empty((size,) + tuple(ct.shape), ct.device)
    check(lib().fheg_expand(par._h, kh, ex, n, size, _dp(ct), _dp(out), _stream()))
    return out


class SecretKey:
    """SecretKey (fhe/src/bfv/keys/secret_key.rs:24-60) resident on the device."""

    def __init__(self, par: BfvParameters, coeffs):
        c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.int64))
        h = c_vp()
        check(lib().fheg_secret_key_create(par._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                           ctypes.byref(h)))
        self._h = h
        self.par = par

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_secret_key_destroy(self._h)
            self._h = None

    def encrypt(self, values, a_ntt, e, level: int = 0, simd: bool = True):
        """try_encrypt with the caller's randomness (secret_key.rs:102-138):
        values [count][N] (< t), a_ntt [count][L][N], e [count][N] (int64)."""
        count = values.shape[0]
        ctx = self.par.context_at_level(level)
        out = empty((count, 2, ctx.L, self.par.degree), values.device)
        check(lib().fheg_encrypt(self._h, level, _dp(values), int(simd), _dp(a_ntt), _dp(e), _dp(out), count,
                                 _stream()))
        return out

    def decrypt(self, ct, level: int = 0, simd: bool = True):
        """try_decrypt + decode (secret_key.rs:200-252, plaintext.rs:337-390):
        [count][parts][L][N] -> [count][N] values mod t."""
        count = ct.shape[0]
        out = empty((count, self.par.degree), ct.device)
        check(lib().fheg_decrypt(self._h, level, ct.shape[1], _dp(ct), int(simd), _dp(out), count, _stream()))
        return out


def ciphertext_add(par: BfvParameters, level: int, a, b):
    """Add<&Ciphertext> (fhe/src/bfv/ops/mod.rs:15-43) on batches."""
    out = empty(a.shape, a.device)
    check(lib().fheg_ciphertext_add(par._h, level, a.shape[1], _dp(a), _dp(b), _dp(out), a.shape[0], _stream()))
    return out


class Multiplicator:
    """bfv::Multiplicator (fhe/src/bfv/ops/mul.rs:21-227)."""

    def __init__(self, handle, par: BfvParameters, keep=()):
        self._h = handle
        self.par = par
        self._keep = list(keep)

    @staticmethod
    def default(rk: RelinearizationKey) -> "Multiplicator":
        """mul.rs:101-130."""
        h = c_vp()
        check(lib().fheg_multiplicator_create_default(rk._h, ctypes.byref(h)))
        return Multiplicator(h, rk.par, [rk])

    @staticmethod
    def new_leveled(lhs: ScalingFactor, rhs: ScalingFactor, extended_basis: Sequence[int], post: ScalingFactor,
                    level: int, par: BfvParameters) -> "Multiplicator":
        """mul.rs:56-98."""
        ws = [_words(x) for x in (lhs.numerator, lhs.denominator, rhs.numerator, rhs.denominator)]
        pn, pd = _words(post.numerator), _words(post.denominator)
        eb = _u64(extended_basis)
        h = c_vp()
        args = []
        for w in ws:
            args += [_ptr(w), len(w)]
        check(lib().fheg_multiplicator_create(par._h, level, *args, _ptr(eb), len(eb), _ptr(pn), len(pn), _ptr(pd),
                                              len(pd), ctypes.byref(h)))
        return Multiplicator(h, par)

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_multiplicator_destroy(self._h)
            self._h = None

    def enable_relinearization(self, rk: RelinearizationKey):
        check(lib().fheg_multiplicator_enable_relinearization(self._h, rk._h))
        self._keep.append(rk)

    def enable_mod_switching(self):
        check(lib().fheg_multiplicator_enable_mod_switching(self._h))

    def output_shape(self):
        parts, level = c_size(0), c_size(0)
        check(lib().fheg_multiplicator_output_shape(self._h, ctypes.byref(parts), ctypes.byref(level)))
        return parts.value, level.value

    def multiply(self, lhs, rhs, out=None, stream: Optional[int] = None):
        """mul.rs:158-227 on batches [count][2][L][N] (device tensors)."""
        if lhs.shape != rhs.shape or lhs.dim() != 4 or lhs.shape[1] != 2:
            raise FhegError(ERR_WRONG_PARTS, "Multiplication can only be performed on ciphertexts of size 2")
        parts, level = self.output_shape()
        count = lhs.shape[0]
        ctx = self.par.context_at_level(level)
        if out is None:
            out = empty((count, parts, ctx.L, ctx.degree), lhs.device)
        check(lib().fheg_multiplicator_multiply(self._h, _dp(lhs), _dp(rhs), _dp(out), count,
                                                _stream() if stream is None else stream))
        return out

    def autotune(self, count: int) -> list:
        """Tunes the per-stage NTT plans on `count`-pair multiplications and
        returns them ([A, C, D, F, F split, tensor split])."""
        out = (ctypes.c_uint32 * 6)()
        check(lib().fheg_multiplicator_autotune(self._h, count, _stream(), out))
        return list(out)

    STAGES = ("A", "B", "C", "D", "E", "F", "G")

    def stage_times(self, lhs, rhs, out) -> dict:
        """One multiplication with events at the stage boundaries: ms per stage."""
        ms = (ctypes.c_float * 7)()
        check(lib().fheg_multiplicator_stage_times(self._h, _dp(lhs), _dp(rhs), _dp(out), lhs.shape[0], _stream(),
                                                   ms))
        return dict(zip(self.STAGES, [float(x) for x in ms]))

    def set_small_plan(self, max_count: int, plan=None):
        """Plan of batches of at most max_count pairs (0 turns it off)."""
        arr = (ctypes.c_uint32 * 6)(*(list(plan or [12, 12, 12, 12, 1, 0]) + [0] * 6)[:6])
        check(lib().fheg_multiplicator_set_small_plan(self._h, max_count, arr))

    @property
    def plan(self) -> list:
        out = (ctypes.c_uint32 * 6)()
        check(lib().fheg_multiplicator_get_plan(self._h, out))
        return list(out)

    @plan.setter
    def plan(self, values):
        values = list(values) + [0] * (6 - len(values))
        arr = (ctypes.c_uint32 * 6)(*values)
        check(lib().fheg_multiplicator_set_plan(self._h, arr))

    def capture(self, lhs, rhs, out) -> "MultiplyGraph":
        """Records multiply(lhs, rhs, out) on these device tensors into a CUDA
        graph (runs it once first)."""
        h = c_vp()
        check(lib().fheg_multiplicator_capture(self._h, _dp(lhs), _dp(rhs), _dp(out), lhs.shape[0],
                                               ctypes.byref(h)))
        return MultiplyGraph(h, [self, lhs, rhs, out])

    def set_host_pipeline(self, chunk: int = 0, streams: int = 3):
        """Chunk size (pairs, 0 = automatic) and stream count of multiply_host."""
        check(lib().fheg_multiplicator_set_host_pipeline(self._h, chunk, streams))

    def multiply_host(self, lhs: np.ndarray, rhs: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
        """End to end from host arrays [count][2][L][N] (u64)."""
        parts, level = self.output_shape()
        count = lhs.shape[0]
        ctx_l = len(self.par.moduli) - level
        if out is None:
            out = np.empty((count, parts, ctx_l, self.par.degree), dtype=np.uint64)
        lhs, rhs = np.ascontiguousarray(lhs, dtype=np.uint64), np.ascontiguousarray(rhs, dtype=np.uint64)
        check(lib().fheg_multiplicator_multiply_host(self._h, _ptr(lhs), _ptr(rhs), _ptr(out), count))
        return out


def multiply_groups(mults: Sequence["Multiplicator"], lhs: Sequence, rhs: Sequence, outs: Sequence = None):
    """Several batched multiplications, one per multiplicator (typically one
    per level), issued together so that they overlap (fheg_multiply_groups)."""
    g = len(mults)
    if outs is None:
        outs = []
        for m, a in zip(mults, lhs):
            parts, level = m.output_shape()
            ctx = m.par.context_at_level(level)
            outs.append(empty((a.shape[0], parts, ctx.L, ctx.degree), a.device))
    mh = (c_vp * g)(*[m._h for m in mults])
    la = (c_vp * g)(*[_dp(a) for a in lhs])
    ra = (c_vp * g)(*[_dp(b) for b in rhs])
    oa = (c_vp * g)(*[_dp(o) for o in outs])
    cn = (c_size * g)(*[a.shape[0] for a in lhs])
    check(lib().fheg_multiply_groups(mh, la, ra, oa, cn, g, _stream()))
    return outs


class MultiplyGraph:
    """A recorded batched multiplication; launch() replays it on the current
    stream. Keeps its multiplicator and buffers alive."""

    def __init__(self, handle, keep):
        self._h = handle
        self._keep = keep

    def launch(self, stream: Optional[int] = None):
        check(lib().fheg_graph_launch(self._h, _stream() if stream is None else stream))

    @property
    def kernels(self) -> int:
        k = c_u64(0)
        check(lib().fheg_graph_kernel_count(self._h, ctypes.byref(k)))
        return k.value

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_graph_destroy(self._h)
            self._h = None


# ---------------------------------------------------------------------------
# Serving runtime (no counterpart in the reference: fhe.rs runs one operation
# per call on the caller's thread).

OP_MUL_RELIN, OP_ROTATE, OP_ADD, OP_SWITCH_DOWN = 0, 1, 2, 3


class Server:
    """Continuous-batching server over a fixed device-memory budget.

    Requests carry host arrays ([2][L][N] u64 ciphertexts); the scheduler
    thread of the library batches pending requests of the same operation and
    parameters, runs them on one of `streams` streams and writes each result
    into its output array. Pinned host arrays (for instance the numpy view of
    a pinned torch tensor) are copied directly; pageable ones through pinned
    staging."""

    def __init__(self, hbm_budget_bytes: int, streams: int = 2, max_batch: int = 64):
        cfg = _ServerConfig(hbm_budget_bytes, streams, max_batch)
        h = c_vp()
        check(lib().fheg_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._live = {}

    def close(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fheg_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _submit(self, op, par, arrays, out_shape, out=None, mult=None, key=None, exponent=0, level=0) -> int:
        arrays = [np.ascontiguousarray(a, dtype=np.uint64) for a in arrays]
        if out is None:
            out = np.empty(out_shape, dtype=np.uint64)
        if tuple(out.shape) != tuple(out_shape) or out.dtype != np.uint64 or not out.flags["C_CONTIGUOUS"]:
            raise FhegError(ERR_INVALID_ARGUMENT, "output array of the wrong shape or type")
        for a in arrays:
            if a.shape[0] != 2:
                raise FhegError(ERR_WRONG_PARTS, "requests take ciphertexts with 2 parts")
        r = _Request(op, par._h, mult._h if mult is not None else None, key._h if key is not None else None,
                     exponent, level, _ptr(arrays[0]), _ptr(arrays[1]) if len(arrays) > 1 else None, _ptr(out))
        rid = c_u64(0)
        check(lib().fheg_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)))
        self._live[rid.value] = (arrays, out)
        return rid.value

    def submit_mul_relin(self, mult: "Multiplicator", lhs, rhs, out=None) -> int:
        parts, level = mult.output_shape()
        shape = (parts, len(mult.par.moduli) - level, mult.par.degree)
        return self._submit(OP_MUL_RELIN, mult.par, [lhs, rhs], shape, out, mult=mult)

    def submit_rotate(self, key: "GaloisKey", ct, out=None) -> int:
        return self._submit(OP_ROTATE, key.par, [ct], ct.shape, out, key=key, exponent=key.exponent)

    def submit_add(self, par: BfvParameters, level: int, a, b, out=None) -> int:
        return self._submit(OP_ADD, par, [a, b], a.shape, out, level=level)

    def submit_switch_down(self, par: BfvParameters, level: int, ct, out=None) -> int:
        shape = (2, ct.shape[1] - 1, ct.shape[2])
        return self._submit(OP_SWITCH_DOWN, par, [ct], shape, out, level=level)

    def wait(self, rid: int, timeout_ms: int = 60000) -> np.ndarray:
        """The request's output; raises FhegError on failure or timeout."""
        st = lib().fheg_server_wait(self._h, rid, timeout_ms)
        if st == ERR_TIMEOUT:
            raise FhegError(st, lib().fheg_last_error().decode())
        _, out = self._live.pop(rid, (None, None))
        check(st)
        return out

    def times(self, rid: int):
        """(submit, start, done) host steady-clock nanoseconds."""
        a, b, c = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        check(lib().fheg_server_request_times(self._h, rid, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def release(self, rid: int):
        check(lib().fheg_server_release(self._h, rid))
        self._live.pop(rid, None)

    def stats(self) -> dict:
        s, c, b, p = c_u64(0), c_u64(0), c_u64(0), c_size(0)
        check(lib().fheg_server_stats(self._h, ctypes.byref(s), ctypes.byref(c), ctypes.byref(b), ctypes.byref(p)))
        return {"submitted": s.value, "completed": c.value, "batches": b.value, "peak_bytes": p.value}
