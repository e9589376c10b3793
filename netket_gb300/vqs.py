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

import torch

from . import _native as nat
from . import kernels as K
from .stats import Stats, _plain_rhat
from .online_stats import not_converged, online_statistics


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
        if chain_length is None:
            chain_length = int(math.ceil(n_samples / sampler.n_chains))
        self.chain_length = int(chain_length)
        self.n_discard_per_chain = 5 if n_discard_per_chain is None else int(n_discard_per_chain)
        self.sampler_state = sampler.init_state(model, self.params_c, sampler_seed)
        self._samples = None
        self._cache = None

    # ---------------------------------------------------------------- parameters
    @property
    def n_samples(self):
        return self.chain_length * self.sampler.n_chains

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
        self._flat.copy_(torch.as_tensor(v, dtype=torch.float64).to(self._flat.device).reshape(-1))
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

    def expect_to_precision(self, op, *, atol=None, rtol=None, max_iter=10_000, max_lag=64):
        """Sample until the standard error of the mean meets ``atol`` (absolute)
        and / or ``rtol`` (relative to |mean|); both must hold when both are given
        (``netket/_src/vqs/expect_to_precision.py:70-164``).  ``op`` is an operator
        or a list / tuple / dict of operators; each has its own ``OnlineStats``
        accumulator (``max_lag`` lags of online autocorrelation), fed with the
        local estimators of every sampling round until it converges, and the
        accumulators are returned in the structure of ``op``.  Later rounds
        discard no sweeps, as in the reference."""
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
        it = 0
        while active and it < max_iter:
            self.sample(n_discard_per_chain=0)
            accs = accumulate(set(active), accs)
            active = [i for i in active if unconverged(accs[i])]
            it += 1
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

    def expect_and_forces(self, op):
        c = self._forward_cache(op)
        n = c["x"].shape[0]
        v = K.center_scale(c["e"], c["stats_dev"][0:1], 1.0 / n)
        F = K.ot_v(c["t"], c["x"], self.N, self.M, v)
        return Stats.from_array(c["stats_dev"].cpu().numpy()), self.model.unflatten(F, self.N, self.M)

    def expect_and_grad(self, op):
        """Energy statistics and grad = 2 Re[(1/n) O^T (E - mean E)]
        (``netket/vqs/mc/mc_state/expect_forces.py:68-111``, ``common.py:103-118``),
        the formula for a hermitian operator; NetKet switches to another one for
        non-hermitian operators (``expect_grad.py:86-128``), not built here."""
        if getattr(op, "is_hermitian", True) is False:
            raise NotImplementedError("expect_and_grad of a non-hermitian operator")
        c = self._forward_cache(op)
        n = c["x"].shape[0]
        v = K.center_scale(c["e"], c["stats_dev"][0:1], 2.0 / n)
        g = K.ot_v(c["t"], c["x"], self.N, self.M, v)
        return Stats.from_array(c["stats_dev"].cpu().numpy()), self.model.unflatten(g, self.N, self.M)

    def __repr__(self):
        return (f"MCState(hilbert={self.hilbert}, sampler={self.sampler}, n_samples={self.n_samples}, "
                f"n_parameters={self.n_parameters}, precision={self.precision})")
