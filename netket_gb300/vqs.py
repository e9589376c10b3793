"""Variational Monte Carlo state (``netket.vqs.MCState``) for the RBM.

``expect``, ``expect_and_grad``, ``expect_and_forces`` and ``local_estimators``
follow ``netket/vqs/mc/mc_state/state.py:521-753`` and the dispatch rules in
``netket/vqs/mc/mc_state/expect*.py``; every array operation is a libvmck
kernel on the GPU.

Precision modes (``precision=``):
  * ``"fp64"``  - every kernel in FP64 (NetKet's numerics; the parity path);
  * ``"fp32"``  - sampler, log-amplitudes and local energies in FP32;
  * ``"mixed"`` - as fp32, with the minSR contraction on tensor cores and the
    solve refined to FP64 (see ``netket_gb300.ngd``).
Statistics and gradient accumulations are FP64 in every mode.
"""
import math
import warnings

import numpy as np
import torch

from . import _native as nat
from . import kernels as K
from .stats import Stats, _plain_rhat
from .online_stats import not_converged, online_statistics


def compute_chain_length(n_chains, n_samples):
    """ceil(n_samples / n_chains), with the reference's warning when that
    rounds the number of samples up (``state.py:60-80``)."""
    if n_samples <= 0:
        raise ValueError(f"Invalid number of samples: n_samples={n_samples}")
    chain_length = int(math.ceil(n_samples / n_chains))
    if chain_length * n_chains != n_samples:
        warnings.warn(f"n_samples={n_samples} does not divide n_chains={n_chains}, increased "
                      f"to {chain_length * n_chains}", UserWarning, stacklevel=3)
    return chain_length


def _derive_seed(seed):
    """A new 64-bit seed from an old one (splitmix64 finaliser)."""
    z = (int(seed) + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def _progress_bar(verbose, total):
    if not verbose:
        return None
    try:
        from tqdm.auto import tqdm
    except ImportError:
        return None
    return tqdm(total=total, desc="expect_to_precision", leave=False, dynamic_ncols=True)


def _check_mutable(mutable):
    if mutable not in (None, False):
        raise NotImplementedError("mutable model collections are not supported (the RBM has "
                                  "none)")


def log_psi_to_array(log_psi, normalize=True):
    """exp(log psi), shifted by max(log psi) and scaled to unit L2 norm when
    ``normalize`` (``netket/nn/utils.py:132-160``)."""
    lp = log_psi.to(torch.float64)
    if normalize:
        lp = lp - lp.max()
    psi = torch.exp(lp)
    if normalize:
        psi = psi / torch.linalg.vector_norm(psi)
    return psi


class MCState:
    def __init__(self, sampler, model, *, n_samples=None, n_samples_per_rank=None,
                 chain_length=None, n_discard_per_chain=None, seed=None, sampler_seed=None,
                 variables=None, precision=None, local_estimator="fused", chunk_size=None,
                 init_fun=None, apply_fun=None, mutable=False, training_kwargs=None):
        # NetKet's remaining MCState arguments (netket/vqs/mc/mc_state/state.py:180-196):
        # chunk_size only bounds memory in NetKet and every kernel here streams its
        # samples, so it is kept and has no effect; the model is the RBM, so custom
        # init / apply functions and mutable collections are refused.
        if init_fun is not None or apply_fun is not None:
            raise NotImplementedError("MCState: custom init_fun / apply_fun are not supported; "
                                      "the model is the RBM")
        if mutable not in (False, None) or training_kwargs:
            raise NotImplementedError("MCState: mutable collections / training_kwargs are not "
                                      "supported")
        self.chunk_size = chunk_size
        nat.require_cuda()
        self.sampler = sampler
        self.model = model
        self.hilbert = sampler.hilbert
        self.N = self.hilbert.size
        self.M = model.n_hidden(self.N)
        if precision is None:
            precision = "fp64" if model.param_dtype == torch.float64 else "fp32"
        if precision not in ("fp64", "fp32", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
        self.precision = precision
        self.compute_dtype = torch.float64 if precision == "fp64" else torch.float32
        if local_estimator not in ("fused", "dense"):
            raise ValueError("local_estimator must be 'fused' or 'dense'")
        self.local_estimator = local_estimator
        seed = 0 if seed is None else int(seed)
        sampler_seed = (seed + 1) if sampler_seed is None else int(sampler_seed)
        self._sampler_seed = sampler_seed
        if variables is not None:
            self._flat = model.flatten(variables.get("params", variables)).to(
                device=nat.device(), dtype=torch.float64).contiguous()
        else:
            self._flat = model.init_flat(seed, self.N)
        self._flat_c = None
        self._version = 0
        self._c_version = -1
        if n_samples is None and chain_length is None:
            n_samples = 1000 if n_samples_per_rank is None else n_samples_per_rank
        self._samples = None
        self._cache = None
        if chain_length is None:
            chain_length = compute_chain_length(sampler.n_chains, n_samples)
        self.chain_length = chain_length
        self.n_discard_per_chain = n_discard_per_chain
        self.sampler_state = sampler.init_state(model, self.params_c, sampler_seed)

    # ---------------------------------------------------------------- parameters
    @property
    def n_samples(self):
        return self.chain_length * self.sampler.n_chains

    @n_samples.setter
    def n_samples(self, n_samples):
        self.chain_length = compute_chain_length(self.sampler.n_chains, n_samples)

    @property
    def n_samples_per_rank(self):
        return self.n_samples  # one device

    @n_samples_per_rank.setter
    def n_samples_per_rank(self, n):
        self.n_samples = n

    @property
    def chain_length(self):
        return self._chain_length

    @chain_length.setter
    def chain_length(self, chain_length):
        """``state.py:436-441``: positive, and the samples are drawn again."""
        if chain_length <= 0:
            raise ValueError(f"Invalid chain length: chain_length={chain_length}")
        self._chain_length = int(chain_length)
        self.reset()

    @property
    def n_discard_per_chain(self):
        return self._n_discard_per_chain

    @n_discard_per_chain.setter
    def n_discard_per_chain(self, n):
        """``state.py:450-468``: None means 5, negative is refused."""
        if n is not None and n < 0:
            raise ValueError(f"Invalid number of discarded samples: n_discard_per_chain={n}")
        self._n_discard_per_chain = 5 if n is None else int(n)

    @property
    def sampler(self):
        return self._sampler

    @sampler.setter
    def sampler(self, sampler):
        """A new sampler gets fresh chains from a seed derived from the state's
        sampler seed; ``n_samples`` is kept, rounded up to the new number of
        chains (``state.py:374-404``)."""
        old = getattr(self, "_sampler", None)
        self._sampler = sampler
        if old is None:
            return
        n_old = self._chain_length * old.n_chains
        self._sampler_seed = _derive_seed(self._sampler_seed)
        self.sampler_state = sampler.init_state(self.model, self.params_c, self._sampler_seed)
        self.n_samples = n_old
        self.reset()

    @property
    def n_parameters(self):
        return self._flat.numel()

    @property
    def parameters(self):
        return self.model.unflatten(self._flat, self.N, self.M)

    @parameters.setter
    def parameters(self, p):
        self.flat_parameters = self.model.flatten(p)

    @property
    def variables(self):
        return {"params": self.parameters}

    @property
    def flat_parameters(self):
        return self._flat

    @flat_parameters.setter
    def flat_parameters(self, v):
        t = v if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v))
        if t.is_complex():
            raise TypeError("MCState: complex parameters are not supported (real RBM path)")
        t = t.to(device=self._flat.device, dtype=torch.float64).reshape(-1)
        if t.numel() != self._flat.numel():
            raise ValueError(f"expected {self._flat.numel()} parameters, got {t.numel()}")
        self._flat.copy_(t)
        self.params_changed()

    def params_changed(self):
        self._version += 1
        self._samples = None
        self._cache = None

    @property
    def params_c(self):
        """Parameters in the compute dtype (cached per parameter version)."""
        if self.compute_dtype == torch.float64:
            return self._flat
        if self._c_version != self._version:
            self._flat_c = K.cast_f32(self._flat, self._flat_c)
            self._c_version = self._version
        return self._flat_c

    # ---------------------------------------------------------------- sampling
    def reset(self):
        self._samples = None
        self._cache = None

    def sample(self, *, chain_length=None, n_samples=None, n_discard_per_chain=None):
        if chain_length is None:
            chain_length = (self.chain_length if n_samples is None
                            else int(math.ceil(n_samples / self.sampler.n_chains)))
        nd = self.n_discard_per_chain if n_discard_per_chain is None else int(n_discard_per_chain)
        p = self.params_c
        self.sampler_state = self.sampler.reset(self.model, p, self.sampler_state)
        self._samples, self.sampler_state = self.sampler.sample(
            self.model, p, state=self.sampler_state, chain_length=chain_length, n_discard=nd)
        self._cache = None
        return self._samples

    @property
    def samples(self):
        if self._samples is None:
            self.sample()
        return self._samples

    def log_value(self, x):
        return self.model.apply(self.params_c, x)

    # ---------------------------------------------------------------- estimators
    def _flat_samples(self):
        s = self.samples
        return s.reshape(-1, self.N)

    def _eloc(self, op, x):
        if self.local_estimator == "dense":
            return K.local_energies_dense(op, self.params_c, x, self.N, self.M)
        return K.local_energies_fused(op, self.params_c, x, self.N, self.M)

    def local_estimators(self, op):
        """E_loc reshaped (n_chains, chain_length), FP64."""
        x = self._flat_samples()
        return self._eloc(op, x).reshape(self.sampler.n_chains, -1)

    def expect(self, op):
        e = self.local_estimators(op)
        return Stats.from_array(K.stats_device(e, _plain_rhat()).cpu().numpy())

    def grad(self, op):
        """The gradient of ``expect(op)`` (``netket/vqs/base.py``: the second
        output of ``expect_and_grad``)."""
        return self.expect_and_grad(op)[1]

    def to_array(self, normalize=True):
        """psi on every basis state, in the order of ``hilbert.all_states()``
        (``netket/nn/utils.py:42-160``): exp(log psi - max log psi), scaled to
        unit norm when ``normalize``.  FP64 device tensor."""
        x = self.hilbert.all_states()
        lp = self.model.apply(self.params_c, x)
        return log_psi_to_array(lp, normalize)

    def expect_to_precision(self, op, *, atol=None, rtol=None, max_iter=10_000, max_lag=64,
                            verbose=True):
        """Sample until the standard error of the mean meets ``atol`` (absolute)
        and / or ``rtol`` (relative to |mean|); both must hold when both are given
        (``netket/_src/vqs/expect_to_precision.py:70-164``).  ``op`` is an operator
        or a list / tuple / dict of operators; each has its own ``OnlineStats``
        accumulator (``max_lag`` lags of online autocorrelation), fed with the
        local estimators of every sampling round until it converges, and the
        accumulators are returned in the structure of ``op``.  Later rounds
        discard no sweeps, as in the reference.  ``verbose`` shows a progress
        bar of the rounds when tqdm is installed."""
        if atol is None and rtol is None:
            raise ValueError("At least one of 'atol' or 'rtol' must be specified.")
        if atol is not None and atol <= 0:
            raise ValueError("atol must be > 0.")
        if rtol is not None and rtol <= 0:
            raise ValueError("rtol must be > 0.")

        if isinstance(op, dict):
            keys, leaves = list(op), list(op.values())
        elif isinstance(op, (list, tuple)):
            keys, leaves = None, list(op)
        else:
            keys, leaves = None, [op]

        def unconverged(acc):
            return not_converged(acc.get_stats(), atol, rtol)

        def accumulate(active, accs):
            return [online_statistics(self.local_estimators(o), a, max_lag=max_lag)
                    if i in active else a for i, (o, a) in enumerate(zip(leaves, accs))]

        self.sample()
        accs = accumulate(set(range(len(leaves))), [None] * len(leaves))
        active = [i for i in range(len(leaves)) if unconverged(accs[i])]
        bar = _progress_bar(verbose, max_iter)
        it = 0
        while active and it < max_iter:
            self.sample(n_discard_per_chain=0)
            accs = accumulate(set(active), accs)
            active = [i for i in active if unconverged(accs[i])]
            it += 1
            if bar is not None:
                bar.set_postfix_str(f"{len(active)} not converged")
                bar.update(1)
        if bar is not None:
            bar.close()
        self.last_precision_rounds = it
        if keys is not None:
            return dict(zip(keys, accs))
        if isinstance(op, (list, tuple)):
            return type(op)(accs)
        return accs[0]

    def _forward_cache(self, op):
        """Samples, tanh(theta), local energies and their device statistics."""
        x = self._flat_samples()
        _, _, t = K.rbm_forward(self.params_c, x, self.N, self.M, want_tanh=True)
        e = self._eloc(op, x)
        st = K.stats_device(e.reshape(self.sampler.n_chains, -1), _plain_rhat())
        self._cache = dict(x=x, t=t, e=e, stats_dev=st, op=op)
        return self._cache

    def expect_and_forces(self, op, *, mutable=None):
        _check_mutable(mutable)
        c = self._forward_cache(op)
        n = c["x"].shape[0]
        v = K.center_scale(c["e"], c["stats_dev"][0:1], 1.0 / n)
        F = K.ot_v(c["t"], c["x"], self.N, self.M, v)
        return Stats.from_array(c["stats_dev"].cpu().numpy()), self.model.unflatten(F, self.N, self.M)

    def expect_and_grad(self, op, *, mutable=None, use_covariance=None):
        """Energy statistics and grad = 2 Re[(1/n) O^T (E - mean E)]
        (``netket/vqs/mc/mc_state/expect_forces.py:68-111``, ``common.py:103-118``):
        the covariance formula, which NetKet uses when ``use_covariance`` is
        True or, by default, when the operator is hermitian
        (``expect_grad.py:42-64``).  Its other formula (``use_covariance=False``,
        the default for a non-hermitian operator) is not built here."""
        _check_mutable(mutable)
        if use_covariance is None:
            use_covariance = getattr(op, "is_hermitian", True)
        if not use_covariance:
            raise NotImplementedError("expect_and_grad with use_covariance=False (the "
                                      "non-hermitian formula) is not implemented")
        c = self._forward_cache(op)
        n = c["x"].shape[0]
        v = K.center_scale(c["e"], c["stats_dev"][0:1], 2.0 / n)
        g = K.ot_v(c["t"], c["x"], self.N, self.M, v)
        return Stats.from_array(c["stats_dev"].cpu().numpy()), self.model.unflatten(g, self.N, self.M)

    def __repr__(self):
        return (f"MCState(hilbert={self.hilbert}, sampler={self.sampler}, n_samples={self.n_samples}, "
                f"n_parameters={self.n_parameters}, precision={self.precision})")
