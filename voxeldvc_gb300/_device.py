"""Device-memory plumbing: torch CUDA tensors as buffers, the current
stream, a per-device scratch pool and numpy <-> device transfers.

Compute never happens here; every kernel is in libvdvc.so.
"""
from __future__ import annotations

import weakref

import numpy as np

from . import _lib

_torch = None


def torch():
    """torch, with a CUDA device required (this package has no CPU path)."""
    global _torch
    if _torch is None:
        import torch as t
        _torch = t
    if not _torch.cuda.is_available():
        raise RuntimeError("voxeldvc_gb300 needs a CUDA GPU (sm_103a); none is visible")
    return _torch


def is_tensor(x) -> bool:
    t = _torch
    if t is None:
        try:
            import torch as t  # noqa: F811
        except ImportError:
            return False
    return isinstance(x, t.Tensor)


_NP2CODE = {np.dtype(np.float32): _lib.F32, np.dtype(np.float64): _lib.F64, np.dtype(np.uint8): _lib.U8,
            np.dtype(np.uint16): _lib.U16, np.dtype(np.int16): _lib.I16, np.dtype(np.int32): _lib.I32}


def np_dtype_of(x) -> np.dtype:
    if is_tensor(x):
        T = torch()
        m = {T.float32: np.float32, T.float64: np.float64, T.uint8: np.uint8, T.bool: np.bool_,
             T.int16: np.int16, T.int32: np.int32, T.int64: np.int64}
        if hasattr(T, "uint16"):
            m[T.uint16] = np.uint16
        return np.dtype(m[x.dtype])
    return np.asarray(x).dtype


def code_of(dtype) -> int:
    d = np.dtype(dtype)
    if d not in _NP2CODE:
        raise ValueError(f"dtype {d} is not supported by libvdvc")
    return _NP2CODE[d]


def torch_dtype(dtype):
    T = torch()
    d = np.dtype(dtype)
    return {np.dtype(np.float32): T.float32, np.dtype(np.float64): T.float64, np.dtype(np.uint8): T.uint8,
            np.dtype(np.bool_): T.bool, np.dtype(np.int16): T.int16, np.dtype(np.int32): T.int32,
            np.dtype(np.int64): T.int64}[d]


def device():
    return torch().device("cuda", torch().cuda.current_device())


def stream() -> int:
    return torch().cuda.current_stream().cuda_stream


def ptr(t) -> int:
    return t.data_ptr() if t is not None else None


def to_device(x, dtype=None):
    """A contiguous CUDA tensor holding x (numpy, list or tensor), cast to
    `dtype` (numpy dtype) when given.  Bool arrays stay 1-byte bool."""
    T = torch()
    if is_tensor(x):
        t = x
        if not t.is_cuda:
            t = t.to(device())
    else:
        a = np.asarray(x)
        if a.dtype == np.uint16:  # torch has no uint16 arithmetic everywhere; ship the bits as int16
            t = T.from_numpy(np.ascontiguousarray(a).view(np.int16)).to(device())
            if dtype is None or np.dtype(dtype) == np.uint16:
                return t
            raise ValueError("uint16 input must be converted by a kernel")
        t = T.from_numpy(np.ascontiguousarray(a)).to(device())
    if dtype is not None and t.dtype != torch_dtype(dtype):
        t = t.to(torch_dtype(dtype))
    return t.contiguous()


def mask_u8(x):
    """Mask as a contiguous 1-byte CUDA tensor (bool or uint8)."""
    T = torch()
    t = to_device(x)
    if t.dtype not in (T.bool, T.uint8):
        t = t != 0
    return t.contiguous()


def empty(n, dtype):
    return torch().empty(n, dtype=torch_dtype(dtype), device=device())


def zeros(n, dtype):
    return torch().zeros(n, dtype=torch_dtype(dtype), device=device())


class _Scratch:
    """Grow-only scratch buffer per (device, stream): work on two streams
    at once (the batch's set-up on a side stream) never shares one."""

    def __init__(self):
        self.bufs = {}

    def get(self, nbytes: int):
        T = torch()
        key = (T.cuda.current_device(), T.cuda.current_stream().cuda_stream)
        b = self.bufs.get(key)
        if b is None or b.numel() < nbytes:
            b = T.empty(max(int(nbytes), 1 << 20), dtype=T.uint8, device=device())
            self.bufs[key] = b
        return b


scratch = _Scratch()


def wants_host(xp) -> bool:
    """The reference's `xp` argument chooses the array type of the results:
    numpy -> host numpy arrays; anything else -> CUDA tensors."""
    return xp is np


class _HostPool:
    """Pinned host buffers for results returned as numpy arrays.

    A device->host copy into freshly allocated pageable memory runs at the
    speed of first-touch page faults (~14 GB/s measured on the GB300 machine,
    against ~190 GB/s into mapped memory), so large results are copied into
    pinned buffers that are reused once the array handed out for them (and
    every view of it, which keeps it alive) is gone.  At most two buffers per
    shape and type are kept; beyond that results use ordinary memory."""

    MIN_BYTES = 1 << 20
    PER_KEY = 2

    def __init__(self):
        self.entries = {}

    def take(self, shape, dtype):
        lst = self.entries.setdefault((tuple(shape), dtype), [])
        for ent in lst:
            if ent[1] is None or ent[1]() is None:
                return ent
        if len(lst) >= self.PER_KEY:
            return None
        ent = [torch().empty(tuple(shape), dtype=dtype, pin_memory=True), None]
        lst.append(ent)
        return ent


host_pool = _HostPool()


def host_result(n, dtype):
    """A pinned host buffer (pool entry) of n elements that a kernel may
    write directly (pinned memory is mapped into the device's address
    space), or None when the pool has none free; hand it out with
    claim_host_result once the writing stream has finished."""
    if n * np.dtype(dtype).itemsize < _HostPool.MIN_BYTES:
        return None
    return host_pool.take((n,), torch_dtype(dtype))


def claim_host_result(ent):
    a = ent[0].numpy()
    ent[1] = weakref.ref(a)
    return a


def out(t, xp):
    if wants_host(xp):
        t = t.detach()
        if t.is_cuda and t.numel() * t.element_size() >= _HostPool.MIN_BYTES:
            ent = host_pool.take(t.shape, t.dtype)
            if ent is not None:
                ent[0].copy_(t, non_blocking=True)
                torch().cuda.current_stream().synchronize()
                a = ent[0].numpy()
                ent[1] = weakref.ref(a)
                return a
        return t.cpu().numpy()
    return t


def scalar_out(x):
    return float(x)
