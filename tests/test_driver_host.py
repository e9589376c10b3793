"""The driver loop, loggers and callbacks on the CPU, with a fake variational
state and a driver whose loss and update are host arithmetic.

Checked against the reference loop (``abstract_variational_driver.py:349-478``,
``callbacks/legacy_wrappers.py``, ``logging/json_log.py``): the hook order, the
legacy-callback rule (a falsy return stops before that step's update), StopRun
from a hook, step rejection, observables every ``step_size`` steps logged before
the loggers read ``log_data``, loggers seeing the pre-update parameters, the
JSON log layout and write cadence, and the stopping callbacks."""
import json
import math
import os

import numpy as np
import pytest
import torch

from netket_gb300 import callbacks as cb
from netket_gb300 import logging as nklog
from netket_gb300.driver import AbstractVariationalDriver
from netket_gb300.models import RBM
from netket_gb300.stats import Stats


class FakeSamplerState:
    acceptance = 0.25


class FakeState:
    N, M = 2, 3

    def __init__(self):
        self.model = RBM(alpha=1)
        self._flat = torch.arange(self.M + self.N * self.M + self.N, dtype=torch.float64)
        self.sampler_state = FakeSamplerState()
        self.resets = 0

    @property
    def flat_parameters(self):
        return self._flat

    @property
    def parameters(self):
        return self.model.unflatten(self._flat, self.N, self.M)

    @property
    def variables(self):
        return {"params": self.parameters}

    def reset(self):
        self.resets += 1

    def expect(self, op):
        return Stats(float(op) * float(self._flat[0]), 0.1, 1.0, 0.0, 1.0)


class FakeSgd:
    def __init__(self, lr):
        self.lr = lr

    def apply(self, state, dp, step):
        state._flat -= self.lr * dp


class FakeDriver(AbstractVariationalDriver):
    """Loss = |params|^2 / 2 with gradient = params; an optional list of losses
    to report instead (to drive the stopping callbacks)."""

    def __init__(self, losses=None, fail_at=None):
        super().__init__(FakeState(), FakeSgd(0.5))
        self.losses, self.fail_at, self.computed = losses, fail_at, []

    def compute_loss_and_update(self):
        s = self.step_count
        if self.fail_at is not None and s == self.fail_at:
            raise RuntimeError("compute failed")
        self.computed.append(s)
        p = self.state._flat
        mean = float(0.5 * (p * p).sum()) if self.losses is None else self.losses[s]
        return Stats(mean, 0.01, 1.0, 0.0, 1.0), p.clone()


class Recorder(cb.AbstractCallback):
    def __init__(self, order=0):
        self.events, self._order = [], order

    @property
    def callback_order(self):
        return self._order

    def on_run_start(self, step, driver):
        self.events.append(("run_start", step))

    def on_step_start(self, step, log_data, driver):
        self.events.append(("step_start", step))

    def on_compute_update_start(self, step, log_data, driver):
        self.events.append(("compute_start", step))

    def on_compute_update_end(self, step, log_data, driver):
        self.events.append(("compute_end", step))

    def before_parameter_update(self, step, log_data, driver):
        self.events.append(("before_update", step, float(driver.state._flat[1]),
                            sorted(log_data)))

    def on_step_end(self, step, log_data, driver):
        self.events.append(("step_end", step, float(driver.state._flat[1])))

    def on_run_end(self, step, driver):
        self.events.append(("run_end", step))

    def on_run_error(self, step, error, driver):
        self.events.append(("run_error", step, type(error).__name__))


def test_run_hook_order_and_runtime_log():
    drv = FakeDriver()
    rec = Recorder()
    log = nklog.RuntimeLog()
    out = drv.run(3, out=log, callback=rec, show_progress=False)
    assert out == (log,) and drv.step_count == 3
    ev = rec.events
    assert ev[0] == ("run_start", 0) and ev[-1] == ("run_end", 3)
    per_step = [e[0] for e in ev[1:6]]
    assert per_step == ["step_start", "compute_start", "compute_end", "before_update", "step_end"]
    # before_update sees the old parameters and the loss in log_data; step_end the new ones
    assert ev[4][2] == 1.0 and ev[4][3] == ["Energy", "acceptance", "wallclock"]
    assert ev[5][2] == 0.5
    assert list(log["Energy"].iters) == [0, 1, 2]
    p0 = np.arange(11.0)
    np.testing.assert_allclose(log["Energy"]["Mean"], [0.5 * (p0 ** 2).sum() * 0.25 ** k
                                                       for k in range(3)])
    np.testing.assert_allclose(log["Energy"].Mean, log.data["Energy"]["Mean"])
    assert set(log["Energy"].keys()) == {"Mean", "Variance", "Sigma", "R_hat", "TauCorr"}
    assert log["Energy"].main_value_name == "Mean"
    np.testing.assert_allclose(np.asarray(log["Energy"]), log["Energy"]["Mean"])
    np.testing.assert_allclose(log["acceptance"]["value"], [0.25] * 3)
    assert np.all(np.diff(log["wallclock"].values) >= 0)
    assert drv.state.resets == 3
    assert drv.run(0, show_progress=False) == ()


def test_legacy_callback_falsy_return_stops_before_the_update(capsys):
    drv = FakeDriver()
    log = nklog.RuntimeLog()
    seen = []

    def stop_at_2(step, log_data, driver):
        seen.append(step)
        return step < 2

    drv.run(10, out=log, callback=stop_at_2, show_progress=False)
    assert seen == [0, 1, 2] and drv.step_count == 2
    np.testing.assert_allclose(drv.state._flat.numpy(), np.arange(11.0) * 0.25)
    assert list(log["Energy"].iters) == [0, 1]
    assert "run stopped before the last step" in capsys.readouterr().out

    drv2 = FakeDriver()
    drv2.run(5, callback=lambda s, d, dr: None, show_progress=False)
    assert drv2.step_count == 0 and drv2.computed == [0]


def test_stop_run_from_step_end_and_error_path():
    class StopAt(cb.AbstractCallback):
        def on_step_end(self, step, log_data, driver):
            if step == 1:
                raise cb.StopRun("enough")

    drv = FakeDriver()
    log = nklog.RuntimeLog()
    rec = Recorder(order=20)
    drv.run(5, out=log, callback=[StopAt(), rec], show_progress=False)
    # the update of step 1 was applied, the counter not advanced, the logger
    # (order 10) never saw step 1 because the stopping callback (order 0) ran first
    assert drv.step_count == 1 and list(log["Energy"].iters) == [0]
    np.testing.assert_allclose(drv.state._flat.numpy(), np.arange(11.0) * 0.25)
    assert rec.events[-1] == ("run_end", 1)

    drv = FakeDriver(fail_at=2)
    rec = Recorder()
    with pytest.raises(RuntimeError, match="compute failed"):
        drv.run(5, callback=rec, show_progress=False)
    assert rec.events[-1] == ("run_error", 2, "RuntimeError") and drv.step_count == 2


def test_rejected_step_is_computed_again():
    class RejectOnce(cb.AbstractCallback):
        def __init__(self):
            self.done = False

        def on_compute_update_end(self, step, log_data, driver):
            if step == 1 and not self.done:
                self.done = True
                return True

    drv = FakeDriver()
    drv.run(3, callback=RejectOnce(), show_progress=False)
    assert drv.computed == [0, 1, 1, 2] and drv.step_count == 3


def test_observables_every_step_size_and_seen_by_loggers():
    drv = FakeDriver()
    log = nklog.RuntimeLog()
    drv.run(5, out=log, obs={"Sx": 2.0, "pair": [1.0, 3.0]}, step_size=2, show_progress=False)
    assert list(log["Sx"].iters) == [0, 2, 4]
    # the observable is estimated before the update: 2 * params[0] of that step
    np.testing.assert_allclose(log["Sx"]["Mean"], [0.0, 0.0, 0.0])
    assert isinstance(log["pair"], list) and list(log["pair"][1].iters) == [0, 2, 4]
    buf = __import__("io").StringIO()
    log.serialize(buf)
    back = nklog.HistoryDict.from_dict(json.loads(buf.getvalue()))
    np.testing.assert_allclose(back["pair"][1]["Mean"], log["pair"][1]["Mean"])
    assert list(log["Energy"].iters) == [0, 1, 2, 3, 4]
    assert drv.estimate({"a": 1.0, "b": (2.0,)})["b"][0].mean == 0.0


def test_json_log(tmp_path):
    prefix = str(tmp_path / "out" / "run")
    drv = FakeDriver()
    drv.run(7, out=prefix, save_params_every=3, write_every=2, show_progress=False)
    with open(prefix + ".log") as f:
        data = json.load(f)
    assert data["Energy"]["iters"] == list(range(7))
    assert set(data["Energy"]) == {"iters", "Mean", "Variance", "Sigma", "R_hat", "TauCorr"}
    assert data["acceptance"]["value"] == [0.25] * 7
    from netket_gb300.serialization import dict_from_bytes
    with open(prefix + ".npz", "rb") as f:
        saved = dict_from_bytes(f.read())
    # flushed at the end of the run with the final parameters
    np.testing.assert_allclose(saved["params"]["visible_bias"],
                               drv.state.parameters["visible_bias"].numpy())
    with pytest.raises(ValueError, match="already exists"):
        nklog.JsonLog(prefix, mode="x")
    with pytest.raises(ValueError, match="Mode not recognized"):
        nklog.JsonLog(prefix, mode="q")
    # append continues the existing log
    lg = nklog.JsonLog(prefix, mode="a")
    drv.run(2, out=lg, show_progress=False)
    with open(prefix + ".log") as f:
        assert json.load(f)["Energy"]["iters"] == list(range(9))
    assert not [p for p in os.listdir(tmp_path / "out") if p.endswith(".tmp") or
                p.endswith(".tmp.json")]
    back = nklog.RuntimeLog.deserialize(prefix + ".log")
    np.testing.assert_allclose(back["Energy"]["Mean"], lg["Energy"]["Mean"])
    assert back._old_step == 8


def test_json_log_write_cadence(tmp_path):
    """The log is written on the first step and then every ``write_every``
    steps; the parameters on the first step and every ``save_params_every``."""
    from netket_gb300.serialization import dict_from_bytes
    prefix = str(tmp_path / "c")
    lg = nklog.JsonLog(prefix, save_params_every=3, write_every=2)
    st = FakeState()
    written, saved = [], []
    for step in range(7):
        lg(step, {"x": float(step)}, st)
        with open(prefix + ".log") as f:
            written.append(json.load(f)["x"]["iters"][-1])
        with open(prefix + ".npz", "rb") as f:
            saved.append(float(dict_from_bytes(f.read())["params"]["Dense"]["bias"][0]))
        st._flat += 1.0
    assert written == [0, 0, 2, 2, 4, 4, 6]
    assert saved == [0.0, 0.0, 0.0, 3.0, 3.0, 3.0, 6.0]


def test_logger_gets_pre_update_parameters(tmp_path):
    seen = []

    class ParamLogger(nklog.RuntimeLog):
        def __call__(self, step, item, variational_state=None):
            seen.append(variational_state.parameters["Dense"]["bias"].clone())
            super().__call__(step, item, variational_state)

    drv = FakeDriver()
    drv.run(2, out=ParamLogger(), show_progress=False)
    np.testing.assert_allclose(seen[0].numpy(), [0.0, 1.0, 2.0])
    np.testing.assert_allclose(seen[1].numpy(), [0.0, 0.5, 1.0])


def test_history_container():
    h = nklog.History(Stats(1.0, 0.1, 2.0, 0.5, 1.01), 3)
    h.append(Stats(2.0, 0.2, 3.0, 0.5, 1.02), 5)
    assert list(h.iters) == [3, 5] and len(h) == 2
    np.testing.assert_allclose(h["Mean"], [1.0, 2.0])
    np.testing.assert_allclose(h.Sigma, [0.1, 0.2])
    assert h[1]["Mean"][0] == 2.0 and list(h[0:1].iters) == [3]
    it = list(h)
    assert it[0] == (3, 1.0)
    rt = nklog.History(json.loads(json.dumps(h.to_dict(), default=nklog._json_default)))
    np.testing.assert_allclose(rt["R_hat"], h["R_hat"])
    with pytest.raises(ValueError, match="differ"):
        h.append(1.0, 6)
    s = nklog.History(torch.tensor(2.5))
    s.append(np.float32(3.5))
    np.testing.assert_allclose(s.values, [2.5, 3.5])
    assert list(s.iters) == [0, 1]
    with pytest.raises(AttributeError):
        _ = s.nothere
    acc = nklog.accum_histories_in_tree(None, {"a": {"b": 1.0}, "c": [1.0, 2.0]}, 0)
    acc = nklog.accum_histories_in_tree(acc, {"a": {"b": 2.0}, "d": 5.0}, 1)
    np.testing.assert_allclose(acc["a/b"]["value"], [1.0, 2.0])
    assert list(acc["d"].iters) == [1] and list(acc["c"][1].iters) == [0]


def test_early_stopping_invalid_loss_and_timeout(capsys):
    losses = [5.0, 4.0, 3.9, 3.95, 3.99, 3.98, 3.97, 1.0]
    drv = FakeDriver(losses=losses)
    drv.run(8, callback=cb.EarlyStopping(min_delta=0.05, patience=2), show_progress=False)
    # improvements at 0, 1, 2; steps 3 and 4 are within min_delta; 5 exceeds patience
    assert drv.step_count == 5

    drv = FakeDriver(losses=[5.0, 4.0, 3.0, 2.0])
    drv.run(4, callback=cb.EarlyStopping(baseline=1.0, patience=1), show_progress=False)
    assert drv.step_count == 1

    drv = FakeDriver(losses=[1.0, math.nan, math.nan, math.nan, 1.0])
    drv.run(5, callback=cb.InvalidLossStopping(patience=2), show_progress=False)
    assert drv.step_count == 2

    drv = FakeDriver(losses=[1.0, math.inf])
    drv.run(2, callback=cb.InvalidLossStopping(), show_progress=False)
    assert drv.step_count == 1

    with pytest.raises(ValueError):
        cb.Timeout(0)
    drv = FakeDriver()
    drv.run(100, callback=cb.Timeout(1e-9), show_progress=False)
    assert drv.step_count == 0
    with pytest.raises(ValueError, match="must be a number"):
        drv.run("10")
    capsys.readouterr()


def test_progress_bar_runs(capsys):
    pytest.importorskip("tqdm")
    drv = FakeDriver()
    drv.run(3)
    assert drv.step_count == 3
    assert "3/3" in capsys.readouterr().err


def test_convergence_stopping():
    """Losses 3, 1, 1, 1, ... smoothed over 2 steps give 3, 2, 1, 1, ...: the
    smoothed loss is at or below the target 1.5 from step 2 on, so with
    patience 1 the counter passes 1 at step 3 and the run stops there."""
    losses = [3.0, 1.0, 1.0, 1.0, 1.0, 1.0]
    drv = FakeDriver(losses=losses)
    drv.run(6, callback=cb.ConvergenceStopping(1.5, smoothing_window=2, patience=1),
            show_progress=False)
    assert drv.step_count == 3
    drv = FakeDriver(losses=[5.0] * 4)
    drv.run(4, callback=cb.ConvergenceStopping(1.0), show_progress=False)
    assert drv.step_count == 4


def test_runtime_log_serialize_to_streams(tmp_path):
    import io
    log = nklog.RuntimeLog()
    for k in range(3):
        log(k, {"Energy": Stats(float(k), 0.1, 1.0, 0.0, 1.0), "x": float(2 * k)})
    t, b = io.StringIO(), io.BytesIO()
    log.serialize(t)
    log.serialize(b)
    assert json.loads(t.getvalue()) == json.loads(b.getvalue().decode())
    assert json.loads(t.getvalue())["x"] == {"iters": [0, 1, 2], "value": [0.0, 2.0, 4.0]}
    log.serialize(str(tmp_path / "run"))
    back = nklog.RuntimeLog.deserialize(str(tmp_path / "run"))
    np.testing.assert_allclose(back["Energy"]["Mean"], [0.0, 1.0, 2.0])
    assert list(log["x"][1:].iters) == [1, 2]


def test_vmc_checks_hilbert_spaces():
    """VMC refuses a Hamiltonian on another Hilbert space (vmc.py:77-84)."""
    import netket_gb300 as nk

    class State:
        hilbert = nk.hilbert.Spin(0.5, 4, total_sz=0)

    H_same = nk.operator.Ising(nk.hilbert.Spin(0.5, 4, total_sz=0), nk.graph.Chain(4), h=1.0)
    nk.driver.VMC(H_same, nk.optimizer.Sgd(0.1), variational_state=State())
    H_other = nk.operator.Ising(nk.hilbert.Spin(0.5, 4), nk.graph.Chain(4), h=1.0)
    with pytest.raises(TypeError, match="hilbert space"):
        nk.driver.VMC(H_other, nk.optimizer.Sgd(0.1), variational_state=State())
