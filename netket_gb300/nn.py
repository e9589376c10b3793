"""``netket.nn`` names a script passes to the RBM: ``log_cosh`` (the RBM's
activation, ``netket/nn/activation.py:78-84``), here a host function on
tensors or arrays; on the device path the kernels evaluate it themselves."""
import math

import numpy as np
import torch


def log_cosh(x):
    """log(cosh(x)) = |x| + log1p(exp(-2|x|)) - log 2, stable for large |x|."""
    if isinstance(x, torch.Tensor):
        a = x.abs()
        return a + torch.log1p(torch.exp(-2.0 * a)) - math.log(2.0)
    a = np.abs(np.asarray(x, dtype=np.float64))
    return a + np.log1p(np.exp(-2.0 * a)) - math.log(2.0)
