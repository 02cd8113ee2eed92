"""The learned pressure warm start's network (C ABI nusifUNet*).

Volumes are CUDA device tensors (torch is only the device-memory plumbing
here), channels-last [B][Z][Y][X][C] float32, every edge a multiple of 4. The
network's forward and backward passes, the loss and the Adam step all run in
the library's own kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def _ptr(t) -> C.c_void_p:
    if not (t.is_cuda and t.is_contiguous() and str(t.dtype) == "torch.float32"):
        raise abi.NusifError("unet: expected a contiguous float32 CUDA tensor")
    return C.c_void_p(t.data_ptr())


class UNet:
    """3-level 3D U-Net, 16/32/64 channels, BF16 weights and activations."""

    def __init__(self, seed: int = 0):
        self.lib = abi.load_library()
        self.handle = self.lib.nusifUNetCreate(seed)
        abi.check(self.lib)
        if not self.handle:
            raise abi.NusifError("nusifUNetCreate failed")
        self.n_params = int(self.lib.nusifUNetParamCount(self.handle))

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self.lib.nusifUNetGetParams(self.handle, out.ctypes.data_as(C.c_void_p), self.n_params)
        abi.check(self.lib)
        return out

    def set_params(self, flat) -> None:
        a = np.ascontiguousarray(flat, dtype=np.float32)
        if a.size != self.n_params:
            raise abi.NusifError(f"unet: {a.size} parameters given, {self.n_params} needed")
        self.lib.nusifUNetSetParams(self.handle, a.ctypes.data_as(C.c_void_p), self.n_params)
        abi.check(self.lib)

    def grads(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self.lib.nusifUNetGetGrads(self.handle, out.ctypes.data_as(C.c_void_p), self.n_params)
        abi.check(self.lib)
        return out

    def set_tensor_core(self, tcgen05: bool) -> None:
        """Convolutions on the tcgen05 kernels (where the volume allows) or on mma.sync."""
        self.lib.nusifUNetSetTensorCore(self.handle, 1 if tcgen05 else 0)
        abi.check(self.lib)

    def forward(self, x):
        """x: [B][Z][Y][X][2] -> [B][Z][Y][X]."""
        import torch
        B, Z, Y, X, _ = x.shape
        out = torch.empty((B, Z, Y, X), dtype=torch.float32, device=x.device)
        self.lib.nusifUNetForward(self.handle, _ptr(x), B, Z, Y, X, _ptr(out))
        abi.check(self.lib)
        return out

    def train_step(self, x, target, lr: float = 1e-3, update: bool = True,
                   want_loss: bool = True) -> float | None:
        B, Z, Y, X, _ = x.shape
        loss = C.c_float()
        self.lib.nusifUNetTrainStep(self.handle, _ptr(x), _ptr(target), B, Z, Y, X,
                                    C.c_float(lr), int(update),
                                    C.byref(loss) if want_loss else None)
        abi.check(self.lib)
        return float(loss.value) if want_loss else None

    def close(self) -> None:
        if self.handle:
            self.lib.nusifUNetFree(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
