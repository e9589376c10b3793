"""Checkpoint / resume of a variational state (``flax.serialization`` as NetKet
uses it: ``netket/vqs/mc/mc_state/state.py:963-1016`` for ``MCState``,
``netket/sampler/metropolis.py:50-74`` for the sampler state).

The state dict has NetKet's structure::

    {"variables": {"params": {"Dense": {"bias", "kernel"}, "visible_bias"}},
     "sampler_state": {"σ", "rng", "n_steps_proc", "n_accepted_proc"},
     "n_samples", "n_discard_per_chain"}

``rng`` holds what this library's counter-based generator needs to continue
the chains' random stream exactly: the Philox key (``seed``) and the proposal
counter.  ``to_bytes`` / ``from_bytes`` mirror ``flax.serialization``'s
functions of the same names; the byte format is a NumPy ``.npz`` archive of the
flattened dict (keys joined with ``/``), which needs nothing beyond NumPy to
read.  Restoring into a state with the same sampler and model continues the
Markov chains bit-for-bit.
"""
import io

import numpy as np
import torch

from . import _native as nat

_SEP = "/"


def _to_numpy(v):
    if isinstance(v, torch.Tensor):
        return v.detach().cpu().numpy()
    return np.asarray(v)


def _flatten(d, prefix=""):
    out = {}
    for k, v in d.items():
        key = f"{prefix}{_SEP}{k}" if prefix else str(k)
        if isinstance(v, dict):
            out.update(_flatten(v, key))
        else:
            out[key] = _to_numpy(v)
    return out


def _unflatten(flat):
    out = {}
    for key, v in flat.items():
        node = out
        parts = key.split(_SEP)
        for p in parts[:-1]:
            node = node.setdefault(p, {})
        node[parts[-1]] = v
    return out


def state_dict(vstate):
    """NetKet-structured state dict of an ``MCState`` (host NumPy arrays)."""
    st = vstate.sampler_state
    params = vstate.model.unflatten(vstate.flat_parameters, vstate.N, vstate.M)
    return {
        "variables": {"params": params},
        "sampler_state": {
            "σ": st.σ,
            "rng": np.array([st.seed, st.counter], dtype=np.uint64),
            "n_steps_proc": np.int64(st.n_steps_proc),
            "n_accepted_proc": st.n_accepted_proc,
        },
        "n_samples": np.int64(vstate.n_samples),
        "n_discard_per_chain": np.int64(vstate.n_discard_per_chain),
    }


def restore_state_dict(vstate, d):
    """Load a state dict produced by ``state_dict`` into ``vstate`` (same model
    and sampler shapes), on the state's device."""
    dev = nat.device()
    p = d["variables"]["params"]
    flat = vstate.model.flatten({
        "Dense": {"bias": torch.as_tensor(np.asarray(p["Dense"]["bias"])),
                  "kernel": torch.as_tensor(np.asarray(p["Dense"]["kernel"]))},
        "visible_bias": torch.as_tensor(np.asarray(p["visible_bias"]))})
    if flat.numel() != vstate.n_parameters:
        raise ValueError(f"parameter count {flat.numel()} does not match the state's "
                         f"{vstate.n_parameters}")
    vstate.flat_parameters = flat
    s = d["sampler_state"]
    st = vstate.sampler_state
    sigma = torch.as_tensor(np.asarray(s["σ"]), dtype=st.σ.dtype, device=dev)
    if sigma.shape != st.σ.shape:
        raise ValueError(f"chain state shape {tuple(sigma.shape)} does not match "
                         f"{tuple(st.σ.shape)}")
    st.σ = sigma.contiguous()
    rng = np.asarray(s["rng"], dtype=np.uint64)
    st.seed, st.counter = int(rng[0]), int(rng[1])
    st.n_steps_proc = int(np.asarray(s["n_steps_proc"]))
    st.n_accepted_proc = torch.as_tensor(np.asarray(s["n_accepted_proc"]), dtype=torch.int64,
                                         device=dev)
    vstate.n_discard_per_chain = int(np.asarray(d["n_discard_per_chain"]))
    vstate.reset()
    return vstate


def to_bytes(vstate):
    buf = io.BytesIO()
    np.savez(buf, **_flatten(state_dict(vstate)))
    return buf.getvalue()


def from_bytes(vstate, data):
    with np.load(io.BytesIO(data), allow_pickle=False) as z:
        flat = {k: z[k] for k in z.files}
    return restore_state_dict(vstate, _unflatten(flat))


def dict_to_bytes(d):
    """The byte format for a plain (nested) dict of arrays."""
    buf = io.BytesIO()
    np.savez(buf, **_flatten(d))
    return buf.getvalue()


def dict_from_bytes(data):
    with np.load(io.BytesIO(data), allow_pickle=False) as z:
        return _unflatten({k: z[k] for k in z.files})
