"""Device-array helpers of the form_factor package."""
import ctypes

import numpy as np
import torch


def dev(a, dtype=torch.float64):
    a = np.ascontiguousarray(a)
    if not a.flags.writeable:  # e.g. a broadcast view: torch wants memory it may write
        a = a.copy()
    return torch.as_tensor(a, dtype=dtype, device="cuda")


def ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
