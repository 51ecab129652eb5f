"""Python side of the learned multigrid initial guess (include/tracer_nn.h).

`Net` wraps the network that libtracer_gpu.so trains and runs with its own
kernels (tcgen05 BF16 convolutions, FP32 Adam); device buffers are passed as
raw pointers (torch tensors are only plumbing for memory).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import load_library, TracerError
from .abi import STATUS

_bound = False


def _lib():
    global _bound
    L = load_library()
    if not _bound:
        vp = C.c_void_p
        L.tcnn_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(vp)]
        L.tcnn_destroy.argtypes = [vp]
        L.tcnn_set_stream.argtypes = [vp, vp]
        L.tcnn_debug_wait_test.argtypes = [vp, C.c_int32]
        L.tcnn_param_count.argtypes = [vp]
        L.tcnn_param_count.restype = C.c_int64
        L.tcnn_get_params.argtypes = [vp, vp]
        L.tcnn_set_params.argtypes = [vp, vp]
        L.tcnn_get_grads.argtypes = [vp, vp]
        L.tcnn_forward.argtypes = [vp, vp, C.c_int32, vp]
        L.tcnn_loss_backward.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(C.c_float)]
        L.tcnn_adam.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float]
        L.tcnn_conv3x3.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, vp, C.c_int32, C.c_int32, vp]
        L.tc_attach_net.argtypes = [vp, vp]
        L.tc_record_solves.argtypes = [vp, vp, vp, C.c_int32]
        L.tc_record_count.argtypes = [vp]
        L.tc_record_count.restype = C.c_int32
        L.tc_guess_stats.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _bound = True
    return L


def _chk(st: int, where: str):
    if st != 0:
        raise TracerError(st, f"{where}: {STATUS.get(st, st)}")


class Net:
    """Encoder-decoder for nb_max images of H x W (H = nz, W = nx)."""

    def __init__(self, nb_max: int, H: int, W: int, seed: int = 1, stream: int | None = None):
        self.L = _lib()
        self.h = C.c_void_p()
        self.nb_max, self.H, self.W = nb_max, H, W
        _chk(self.L.tcnn_create(nb_max, H, W, seed, C.byref(self.h)), "tcnn_create")
        if stream is not None:
            _chk(self.L.tcnn_set_stream(self.h, C.c_void_p(stream)), "tcnn_set_stream")

    def close(self):
        if self.h:
            self.L.tcnn_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nparams(self) -> int:
        return int(self.L.tcnn_param_count(self.h))

    def get_params(self) -> np.ndarray:
        a = np.empty(self.nparams, dtype=np.float32)
        _chk(self.L.tcnn_get_params(self.h, a.ctypes.data_as(C.c_void_p)), "tcnn_get_params")
        return a

    def set_params(self, a: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float32)
        assert a.size == self.nparams
        _chk(self.L.tcnn_set_params(self.h, a.ctypes.data_as(C.c_void_p)), "tcnn_set_params")

    def get_grads(self) -> np.ndarray:
        a = np.empty(self.nparams, dtype=np.float32)
        _chk(self.L.tcnn_get_grads(self.h, a.ctypes.data_as(C.c_void_p)), "tcnn_get_grads")
        return a

    def forward(self, raw_ptr: int, nb: int, out_ptr: int):
        _chk(self.L.tcnn_forward(self.h, C.c_void_p(raw_ptr), nb, C.c_void_p(out_ptr)), "tcnn_forward")

    def loss_backward(self, raw_ptr: int, sf_new_ptr: int, nb: int) -> float:
        loss = C.c_float(0)
        _chk(self.L.tcnn_loss_backward(self.h, C.c_void_p(raw_ptr), C.c_void_p(sf_new_ptr), nb, C.byref(loss)),
             "tcnn_loss_backward")
        return float(loss.value)

    def debug_wait_test(self, on: bool):
        """Timeout-path test: every convolution waits on a word nothing sets (tcnn_debug_wait_test)."""
        _chk(self.L.tcnn_debug_wait_test(self.h, 1 if on else 0), "tcnn_debug_wait_test")

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        _chk(self.L.tcnn_adam(self.h, lr, beta1, beta2, eps), "tcnn_adam")

    def save(self, path: str):
        np.save(path, self.get_params())

    def load(self, path: str):
        self.set_params(np.load(path))


def conv3x3(x_ptr: int, nb: int, H: int, W: int, cin: int, w_ptr: int, b_ptr: int, cout: int, relu: bool,
            y_ptr: int):
    """One network convolution on device buffers (BF16 NHWC in/out)."""
    _chk(_lib().tcnn_conv3x3(C.c_void_p(x_ptr), nb, H, W, cin, C.c_void_p(w_ptr), C.c_void_p(b_ptr), cout,
                             1 if relu else 0, C.c_void_p(y_ptr)), "tcnn_conv3x3")


def attach(sim, net: Net | None):
    _chk(_lib().tc_attach_net(sim.h, net.h if net is not None else None), "tc_attach_net")


def record_solves(sim, raw_ptr: int, sf_ptr: int, capacity: int):
    _chk(_lib().tc_record_solves(sim.h, C.c_void_p(raw_ptr), C.c_void_p(sf_ptr), capacity), "tc_record_solves")


def record_count(sim) -> int:
    return int(_lib().tc_record_count(sim.h))


def guess_stats(sim) -> tuple[int, int]:
    u, o = C.c_int64(0), C.c_int64(0)
    _chk(_lib().tc_guess_stats(sim.h, C.byref(u), C.byref(o)), "tc_guess_stats")
    return int(u.value), int(o.value)
