"""Loggers for the driver loop (``netket.logging``): ``RuntimeLog`` and ``JsonLog``,
over the time-series container ``History``.

A logger is called as ``logger(step, log_data, variational_state)`` after each
accepted step and ``logger.flush(variational_state)`` when a run ends
(``netket/_src/logging/runtime_log.py:49-58``, ``json_log.py:129-160``).  The
logged tree is accumulated leaf by leaf (``netket/utils/history/accum.py:84-175``):
dicts, lists and tuples are walked; an object with ``to_compound`` (``Stats``)
is one leaf whose fields (``Mean``, ``Variance``, ``Sigma``, ``R_hat``,
``TauCorr``) share a time axis; an object with only ``to_dict`` is walked as
its dict; anything else (a number, an array, a tensor) is a leaf named
``value``.  So ``log["Energy"]["Mean"]``, ``log["Energy"].Mean`` and
``log["Energy"].iters`` read as in NetKet.

``JsonLog`` writes the accumulated tree as JSON to ``<prefix>.log`` (the
layout of ``History.to_dict``: ``{"Energy": {"iters": [...], "Mean": [...],
...}}``) and the variational state's variables to ``<prefix>.npz`` in the byte
format of ``netket_gb300.serialization`` (NetKet writes flax msgpack to
``<prefix>.mpack``; flax is not a dependency here).
"""
import json
import os
import time
from pathlib import Path

import numpy as np
import torch


def _host(v):
    """A logged leaf value as a host NumPy scalar / array."""
    if isinstance(v, torch.Tensor):
        v = v.detach().cpu().numpy()
    a = np.asarray(v)
    return a[()] if a.ndim == 0 else a


def _fields(value):
    """(main field name, {field: value}) of one logged leaf."""
    if hasattr(value, "to_compound"):
        main, d = value.to_compound()
        return main, dict(d)
    if hasattr(value, "to_dict") and not isinstance(value, (dict, History)):
        d = dict(value.to_dict())
        return (next(iter(d)) if len(d) == 1 else None), d
    if isinstance(value, dict):
        return (next(iter(value)) if len(value) == 1 else None), dict(value)
    return "value", {"value": value}


class History:
    """A set of time series sharing one time axis (``netket.utils.history.History``):
    ``iters`` is the time axis, ``h[key]`` / ``h.key`` a series as an array,
    ``values`` the main series (``Mean`` for ``Stats``, ``value`` for a number)."""

    __slots__ = ("_iters", "_series", "_main")

    def __init__(self, values=None, iters=None, main_value_name=None):
        self._iters, self._series, self._main = [], {}, main_value_name
        if values is None:
            return
        if isinstance(values, dict) and "iters" in values and iters is None:
            # a History previously turned into a dict (JSON round trip)
            its = list(values["iters"])
            self._iters = its
            for k, v in values.items():
                if k != "iters":
                    self._series[k] = list(v)
            if self._main is None and len(self._series) == 1:
                self._main = next(iter(self._series))
            return
        self.append(values, 0 if iters is None else iters)

    def append(self, val, it=None):
        main, d = _fields(val)
        if "iters" in d:
            raise ValueError("cannot have a field called iters")
        if not self._iters:
            self._series = {k: [] for k in d}
            if self._main is None:
                self._main = main
        elif set(d) != set(self._series):
            raise ValueError(f"logged fields {sorted(d)} differ from the history's "
                             f"{sorted(self._series)}")
        if it is None:
            it = (self._iters[-1] + 1) if self._iters else 0
        self._iters.append(it)
        for k, v in d.items():
            self._series[k].append(_host(v))

    @property
    def iters(self):
        return np.asarray(self._iters)

    @property
    def main_value_name(self):
        return self._main

    @property
    def values(self):
        if self._main is None:
            raise ValueError("No main value defined for this history object.")
        return self[self._main]

    def keys(self):
        return list(self._series)

    def __contains__(self, key):
        return key == "iters" or key in self._series

    def __len__(self):
        return len(self._iters)

    def __getitem__(self, key):
        if isinstance(key, slice) or (isinstance(key, int) and key not in self._series):
            idx = range(len(self._iters))[key]
            idx = [idx] if isinstance(idx, int) else list(idx)
            h = History(main_value_name=self._main)
            h._iters = [self._iters[i] for i in idx]
            h._series = {k: [v[i] for i in idx] for k, v in self._series.items()}
            return h
        if key == "iters":
            return self.iters
        return np.asarray(self._series[key])

    def __getattr__(self, attr):
        if attr.startswith("_"):
            raise AttributeError(attr)
        if attr in self._series:
            return np.asarray(self._series[attr])
        raise AttributeError(f"History object has no attribute {attr}. "
                             f"Available keys are {self.keys()}.")

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.values, dtype=dtype)

    def __iter__(self):
        return iter(zip(self.iters, self.values))

    def get(self):
        return self.iters, self.values

    def to_dict(self):
        out = {"iters": self.iters}
        for k in self._series:
            out[k] = np.asarray(self._series[k])
        return out

    def __repr__(self):
        return f"History(keys={self.keys()}, n_iters={len(self)})"


class HistoryDict(dict):
    """A nested dict of ``History`` leaves; ``d["a/b"]`` is ``d["a"]["b"]``."""

    def __getitem__(self, key):
        if isinstance(key, str) and "/" in key and not dict.__contains__(self, key):
            node = self
            for part in key.split("/"):
                node = node[part]
            return node
        return dict.__getitem__(self, key)

    def to_dict(self):
        return {k: v.to_dict() for k, v in self.items()}

    @classmethod
    def from_dict(cls, d):
        out = cls()
        for k, v in d.items():
            out[k] = cls._node(v)
        return out

    @classmethod
    def _node(cls, v):
        if isinstance(v, dict):
            return History(v) if "iters" in v else cls.from_dict(v)
        if isinstance(v, list):
            return [cls._node(x) for x in v]
        raise ValueError(f"not a logged history: {v!r}")


def accum_histories_in_tree(acc, tree, step):
    """Append the leaves of ``tree`` to the histories in ``acc`` (created where
    missing), walking dicts / lists / tuples and objects with only ``to_dict``."""
    if tree is None:
        return acc
    if isinstance(tree, dict) or (hasattr(tree, "to_dict") and not hasattr(tree, "to_compound")
                                  and not isinstance(tree, History)):
        d = tree if isinstance(tree, dict) else tree.to_dict()
        if not d:
            return acc
        acc = HistoryDict() if acc is None else acc
        for k, v in d.items():
            r = accum_histories_in_tree(acc.get(k), v, step)
            if r is not None:
                acc[k] = r
        return acc
    if isinstance(tree, (list, tuple)):
        if not tree:
            return acc
        acc = [None] * len(tree) if acc is None else list(acc)
        return type(tree)(accum_histories_in_tree(a, t, step) for a, t in zip(acc, tree))
    if acc is None:
        return History(tree, step)
    acc.append(tree, step)
    return acc


def _json_default(obj):
    if isinstance(obj, (History, HistoryDict)):
        return obj.to_dict()
    if isinstance(obj, np.ndarray):
        if np.iscomplexobj(obj):
            return {"real": obj.real.tolist(), "imag": obj.imag.tolist()}
        return obj.tolist()
    if isinstance(obj, np.generic):
        return obj.item()
    if isinstance(obj, complex):
        return {"real": obj.real, "imag": obj.imag}
    if hasattr(obj, "to_dict"):
        return obj.to_dict()
    raise TypeError(f"cannot serialise {type(obj).__name__}")


class RuntimeLog:
    """Accumulates the logged tree in memory (``runtime_log.py:30-180``)."""

    def __init__(self):
        self._data = HistoryDict()
        self._old_step = 0

    def __call__(self, step, item, variational_state=None):
        self._data = accum_histories_in_tree(self._data, item, step)
        self._old_step = step

    @property
    def data(self):
        return self._data

    def __getitem__(self, key):
        return self._data[key]

    def flush(self, variational_state=None):
        pass

    def serialize(self, path):
        """Write ``data`` as JSON; a path without ``.log`` / ``.json`` gets ``.json``."""
        if isinstance(path, (str, Path)):
            path = Path(path)
            if not path.name.endswith((".log", ".json")):
                path = path.parent / (path.name + ".json")
            with open(path, "w") as f:
                json.dump(self._data, f, default=_json_default)
        else:
            text = json.dumps(self._data, default=_json_default)
            try:
                path.write(text)
            except TypeError:  # a binary stream
                path.write(text.encode())

    @classmethod
    def deserialize(cls, path):
        path = Path(path)
        if not path.name.endswith((".log", ".json")):
            path = path.parent / (path.name + ".json")
        with open(path) as f:
            raw = json.load(f)
        log = cls()
        log._data = HistoryDict.from_dict(raw)

        def last(d):
            m = 0
            for v in d.values():
                if isinstance(v, History):
                    m = max(m, int(v.iters[-1])) if len(v) else m
                else:
                    m = max(m, last(v))
            return m

        log._old_step = last(log._data)
        return log

    def __repr__(self):
        return f"RuntimeLog():\n keys = {list(self._data)}"


class JsonLog(RuntimeLog):
    """``RuntimeLog`` that also writes ``<prefix>.log`` every ``write_every``
    steps and the variables to ``<prefix>.npz`` every ``save_params_every``
    steps (``json_log.py:52-230``; without the time-based autoflush).  ``mode``:
    ``"write"``/``"w"`` overwrites, ``"append"``/``"a"`` continues an existing
    log, ``"fail"``/``"x"`` refuses an existing one."""

    def __init__(self, output_prefix, mode="write", save_params_every=50, write_every=50,
                 save_params=True):
        super().__init__()
        mode = {"w": "write", "a": "append", "x": "fail"}.get(mode, mode)
        if mode not in ("write", "append", "fail"):
            raise ValueError("Mode not recognized: should be one of `[w]rite`, `[a]ppend` or "
                             "`[x]`(fail).")
        prefix = str(output_prefix)
        exists = os.path.exists(prefix + ".log") or os.path.exists(prefix + ".npz")
        if exists and mode == "fail":
            raise ValueError("Output file already exists. Either delete it manually or "
                             "change `output_prefix`.")
        d = os.path.dirname(prefix)
        if d:
            os.makedirs(d, exist_ok=True)
        self._prefix, self._file_mode = prefix, mode
        self._write_every, self._save_params_every = int(write_every), int(save_params_every)
        self._save_params = save_params
        self._unwritten = 0
        self._unsaved = 0
        self._flush_log_time = 0.0
        self._flush_pars_time = 0.0
        if mode == "append" and os.path.exists(prefix + ".log"):
            old = RuntimeLog.deserialize(prefix + ".log")
            self._data, self._old_step = old._data, old._old_step

    def __call__(self, step, item, variational_state=None):
        super().__call__(step, item, variational_state)
        if self._unwritten % self._write_every == 0:
            self._flush_log()
        if self._unsaved % self._save_params_every == 0:
            self._flush_params(variational_state)
        self._unwritten += 1
        self._unsaved += 1

    def _flush_log(self):
        t = time.perf_counter()
        tmp = f"{self._prefix}.log.{os.getpid()}.tmp"
        self.serialize(tmp + ".json")
        os.replace(tmp + ".json", self._prefix + ".log")
        self._flush_log_time += time.perf_counter() - t
        self._unwritten = 0

    def _flush_params(self, variational_state):
        if not self._save_params or variational_state is None:
            return
        from .serialization import dict_to_bytes
        t = time.perf_counter()
        data = dict_to_bytes(variational_state.variables)
        with open(self._prefix + ".npz", "wb") as f:
            f.write(data)
        self._flush_pars_time += time.perf_counter() - t
        self._unsaved = 0

    def flush(self, variational_state=None):
        self._flush_log()
        if variational_state is not None:
            self._flush_params(variational_state)

    def __repr__(self):
        return (f"JsonLog('{self._prefix}', mode={self._file_mode})\n  Runtime cost:"
                f"\n  \tLog:    {self._flush_log_time}\n  \tParams: {self._flush_pars_time}")
