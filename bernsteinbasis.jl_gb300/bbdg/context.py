"""Per-device library contexts and tensor plumbing (torch supplies memory and streams)."""
from __future__ import annotations

import ctypes
import threading

import torch

from . import _lib

_contexts: dict = {}
_ctx_lock = threading.Lock()


class Context:
    """Owns one bb_ctx (tables, reduction scratch) on one CUDA device."""

    def __init__(self, device: int = 0):
        L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(L.bb_ctx_create(int(device), ctypes.byref(h)), None,
                   f"bb_ctx_create(device={device})")
        self.handle = h
        self.device = int(device)

    def last_error(self) -> str:
        e = _lib.load().bb_ctx_last_error(self.handle)
        return e.decode() if e else ""

    def launch_count(self) -> int:
        return int(_lib.load().bb_ctx_launch_count(self.handle))

    def check(self, rc: int, what: str = "") -> None:
        _lib.check(rc, self.handle, what)

    def set_wait_limit(self, polls: int = 0) -> None:
        """Polls before a device-side mbarrier wait gives up (0: the default, about 1 s)."""
        self.check(_lib.load().bb_ctx_set_wait_limit(self.handle, int(polls)),
                   "bb_ctx_set_wait_limit")

    def set_test_fault(self, mode: int) -> None:
        """Test only: 1 leaves one bulk copy out so that a bounded wait runs out; 0 = off."""
        self.check(_lib.load().bb_ctx_set_test_fault(self.handle, int(mode)),
                   "bb_ctx_set_test_fault")

    def device_status(self, stream=None) -> int:
        """Reads and clears the context's device status word (GEMM and closure kernels)."""
        out = ctypes.c_int(0)
        self.check(_lib.load().bb_device_status(self.handle, stream_handle(stream),
                                                ctypes.byref(out)), "bb_device_status")
        return out.value

    def close(self) -> None:
        if self.handle:
            _lib.load().bb_ctx_destroy(self.handle)
            self.handle = None


def get_context(device=None) -> Context:
    """The shared context of a CUDA device (created on first use)."""
    if device is None:
        device = torch.cuda.current_device()
    if isinstance(device, torch.device):
        device = device.index if device.index is not None else torch.cuda.current_device()
    with _ctx_lock:
        ctx = _contexts.get(int(device))
        if ctx is None:
            ctx = Context(int(device))
            _contexts[int(device)] = ctx
        return ctx


def dtype_code(t: torch.dtype) -> int:
    if t == torch.float32:
        return _lib.BB_F32
    if t == torch.float64:
        return _lib.BB_F64
    raise TypeError(f"unsupported dtype {t}; use torch.float32 or torch.float64")


def ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def stream_handle(stream=None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def require_cuda(*tensors) -> None:
    for t in tensors:
        if not isinstance(t, torch.Tensor):
            raise TypeError("expected a torch.Tensor")
        if not t.is_cuda:
            raise ValueError("tensor must live on a CUDA device (there is no CPU path)")
        if not t.is_contiguous():
            raise ValueError("tensor must be contiguous")
