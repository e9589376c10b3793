"""The RBM (``netket.models.RBM``, ``netket/models/rbm.py:33-81``).

logpsi(x) = sum_j log_cosh(b_j + sum_i x_i W_ij) + sum_i a_i x_i.

Parameters follow NetKet's pytree ``{"Dense": {"bias": (M,), "kernel": (N, M)},
"visible_bias": (N,)}`` and its ravel order (sorted keys): bias, kernel
(row-major), visible_bias.  On the device they live in one flat buffer in that
order, which is the layout every kernel takes.
"""
import numpy as np
import torch

from . import _native as nat


def _real_param_dtype(dt):
    """torch.float64 / torch.float32 from any spelling NetKet scripts use
    (``float``, ``np.float64``, ``"float32"``, a torch dtype); complex and
    other types are refused."""
    if isinstance(dt, torch.dtype):
        if dt in (torch.float64, torch.float32):
            return dt
        raise NotImplementedError(f"RBM: param_dtype {dt} is not supported (float64 / float32)")
    try:
        npdt = np.dtype(dt)
    except TypeError as err:
        raise ValueError(f"RBM: param_dtype {dt!r} is not a dtype") from err
    if npdt == np.float64:
        return torch.float64
    if npdt == np.float32:
        return torch.float32
    if np.issubdtype(npdt, np.complexfloating):
        raise NotImplementedError("RBM: complex parameters are not supported (real RBM path)")
    raise NotImplementedError(f"RBM: param_dtype {npdt} is not supported (float64 / float32)")


class RBM:
    """``alpha``, ``param_dtype`` (float64 or float32, any spelling) and the two
    bias switches as in ``netket/models/rbm.py:33-56``; the activation is
    log_cosh.  Parameters start Normal(0, std) per leaf (NetKet's
    ``normal(stddev=0.01)`` initialisers); ``*_init_std`` set the three
    standard deviations.  JAX initialiser functions, another activation and
    ``precision`` have no meaning here and are refused."""

    def __init__(self, alpha=1, param_dtype=torch.float64, use_hidden_bias=True,
                 use_visible_bias=True, kernel_init_std=0.01, hidden_bias_init_std=0.01,
                 visible_bias_init_std=0.01, *, activation=None, precision=None,
                 kernel_init=None, hidden_bias_init=None, visible_bias_init=None):
        if not (use_hidden_bias and use_visible_bias):
            raise NotImplementedError("the RBM kernels take both biases")
        if activation is not None and getattr(activation, "__name__", "") != "log_cosh":
            raise NotImplementedError("RBM: only the log_cosh activation is implemented")
        if precision is not None:
            raise NotImplementedError("RBM: precision= selects JAX matmul precision; use "
                                      "MCState(precision=...) here")
        if any(f is not None for f in (kernel_init, hidden_bias_init, visible_bias_init)):
            raise NotImplementedError("RBM: JAX initialiser functions are not supported; "
                                      "use kernel_init_std / hidden_bias_init_std / "
                                      "visible_bias_init_std")
        if alpha <= 0:
            raise ValueError(f"RBM: alpha must be positive, got {alpha}")
        self.alpha = alpha
        self.param_dtype = _real_param_dtype(param_dtype)
        self.stds = (hidden_bias_init_std, kernel_init_std, visible_bias_init_std)

    def n_hidden(self, N):
        return int(self.alpha * N)

    def n_parameters(self, N):
        M = self.n_hidden(N)
        return M + N * M + N

    def init_flat(self, seed, N):
        """Flat FP64 parameters, each leaf ~ Normal(0, std) (``rbm.py:29``)."""
        M = self.n_hidden(N)
        g = torch.Generator().manual_seed(int(seed))
        sb, sk, sv = self.stds
        flat = torch.cat([torch.randn(M, generator=g, dtype=torch.float64) * sb,
                          torch.randn(N * M, generator=g, dtype=torch.float64) * sk,
                          torch.randn(N, generator=g, dtype=torch.float64) * sv])
        if self.param_dtype == torch.float32:
            flat = flat.to(torch.float32).to(torch.float64)
        return flat.to(nat.device())

    @staticmethod
    def unflatten(flat, N, M):
        return {"Dense": {"bias": flat[:M], "kernel": flat[M:M + N * M].view(N, M)},
                "visible_bias": flat[M + N * M:]}

    @staticmethod
    def flatten(params):
        """The flat vector [bias | kernel (row-major) | visible_bias] of a
        parameter pytree whose leaves are tensors or array-likes (NumPy arrays
        loaded from a file, lists); complex leaves are refused."""
        leaves = [params["Dense"]["bias"], params["Dense"]["kernel"], params["visible_bias"]]
        out = []
        for leaf in leaves:
            t = leaf if isinstance(leaf, torch.Tensor) else torch.as_tensor(np.asarray(leaf))
            if t.is_complex():
                raise TypeError("RBM: complex parameters are not supported (real RBM path)")
            out.append(t.reshape(-1))
        if len({t.device for t in out}) > 1:
            out = [t.to(out[0].device) for t in out]
        return torch.cat(out)

    @staticmethod
    def sizes_from_flat(P, N):
        M = (P - N) // (N + 1)
        if M + N * M + N != P:
            raise ValueError("parameter vector does not match an RBM on N sites")
        return M

    def apply(self, flat, x, dtype=None):
        """logpsi(x) for x (..., N) int8 with flat parameters (device)."""
        dtype = dtype or flat.dtype
        x = x.to(device=flat.device, dtype=torch.int8)
        N = x.shape[-1]
        M = self.sizes_from_flat(flat.numel(), N)
        p = flat.to(dtype).contiguous()
        x2 = x.reshape(-1, N).contiguous()
        out = torch.empty(x2.shape[0], dtype=dtype, device=flat.device)
        nat.check(nat.lib().vmck_rbm_logpsi(nat.stream(), nat.dtype_code(dtype), nat.ptr(p), N, M,
                                            nat.ptr(x2), x2.shape[0], nat.ptr(out), None, None))
        return out.reshape(x.shape[:-1])

    def __repr__(self):
        return f"RBM(alpha={self.alpha}, param_dtype={self.param_dtype})"

