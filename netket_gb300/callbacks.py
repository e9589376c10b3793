"""Callbacks for the driver loop (``netket.callbacks``).

Hooks and their order within one step follow
``netket/_src/driver/abstract_variational_driver.py:420-478`` and
``netket/_src/callbacks/base.py``: ``on_run_start``; per step
``on_step_start``, ``on_compute_update_start``, ``on_compute_update_end``
(returning True rejects the step, which is computed again),
``before_parameter_update`` (the loss is in ``log_data``, the parameters are
still the step's), ``on_step_end`` (after the update, before the step counter
moves); ``on_run_end`` or ``on_run_error``.  Raising ``StopRun`` from any hook
ends the run normally.  Callbacks run in ``callback_order`` (0 by default,
10 for loggers, so observables are in ``log_data`` before a logger reads it).

A plain function ``f(step, log_data, driver)`` is a legacy callback: it is
called at ``before_parameter_update`` and a falsy return stops the run before
that step's parameter update (``legacy_wrappers.py:16-33``).
"""
import time
from collections import deque

import numpy as np


class StopRun(Exception):
    """Raised from a callback hook to end the run (``callbacks/base.py``)."""


class AbstractCallback:
    @property
    def callback_order(self):
        return 0

    def on_run_start(self, step, driver):
        pass

    def on_step_start(self, step, log_data, driver):
        pass

    def on_compute_update_start(self, step, log_data, driver):
        pass

    def on_compute_update_end(self, step, log_data, driver):
        return False

    def before_parameter_update(self, step, log_data, driver):
        pass

    def on_step_end(self, step, log_data, driver):
        pass

    def on_run_end(self, step, driver):
        pass

    def on_run_error(self, step, error, driver):
        pass


class CallbackList(AbstractCallback):
    """Callbacks sorted by ``callback_order`` (stable), called in turn."""

    def __init__(self, callbacks=()):
        if isinstance(callbacks, AbstractCallback):
            callbacks = (callbacks,)
        self.callbacks = tuple(sorted(callbacks, key=lambda c: c.callback_order))

    def on_run_start(self, step, driver):
        for c in self.callbacks:
            c.on_run_start(step, driver)

    def on_step_start(self, step, log_data, driver):
        for c in self.callbacks:
            c.on_step_start(step, log_data, driver)

    def on_compute_update_start(self, step, log_data, driver):
        for c in self.callbacks:
            c.on_compute_update_start(step, log_data, driver)

    def on_compute_update_end(self, step, log_data, driver):
        reject = False
        for c in self.callbacks:
            if c.on_compute_update_end(step, log_data, driver) is True:
                reject = True
        return reject

    def before_parameter_update(self, step, log_data, driver):
        for c in self.callbacks:
            c.before_parameter_update(step, log_data, driver)

    def on_step_end(self, step, log_data, driver):
        for c in self.callbacks:
            c.on_step_end(step, log_data, driver)

    def on_run_end(self, step, driver):
        for c in self.callbacks:
            c.on_run_end(step, driver)

    def on_run_error(self, step, error, driver):
        for c in self.callbacks:
            c.on_run_error(step, error, driver)


class LegacyCallbackWrapper(AbstractCallback):
    def __init__(self, callback):
        self.callback = callback

    def before_parameter_update(self, step, log_data, driver):
        if not self.callback(step, log_data, driver):
            raise StopRun(f"Legacy callback {self.callback} requested to stop the run.")


class LegacyLoggerWrapper(AbstractCallback):
    """A logger called at the end of each step with a snapshot of the state
    taken before the parameter update, and flushed when the run ends."""

    def __init__(self, logger):
        self.logger = logger
        self._vstate = None

    @property
    def callback_order(self):
        return 10

    def before_parameter_update(self, step, log_data, driver):
        self._vstate = _StateSnapshot(driver.state)

    def on_step_end(self, step, log_data, driver):
        self.logger(step, log_data, self._vstate)
        self._vstate = None

    def on_run_end(self, step, driver):
        self.logger.flush(driver.state)
        self._vstate = None

    def on_run_error(self, step, error, driver):
        self.logger.flush(driver.state)
        self._vstate = None


class _StateSnapshot:
    """The variables of a variational state as they were when the snapshot was
    taken (NetKet copies the immutable state; the parameters here live in a
    device buffer that the update overwrites, so they are copied)."""

    def __init__(self, vstate):
        self._vstate = vstate
        self._flat = vstate.flat_parameters.clone()

    @property
    def parameters(self):
        v = self._vstate
        return v.model.unflatten(self._flat, v.N, v.M)

    @property
    def variables(self):
        return {"params": self.parameters}

    def __getattr__(self, attr):
        return getattr(self._vstate, attr)


def maybe_wrap_legacy_callback(callback):
    if isinstance(callback, AbstractCallback):
        return callback
    return LegacyCallbackWrapper(callback)


class ObservableCallback(AbstractCallback):
    """Adds ``driver.estimate(observables)`` to ``log_data`` every ``interval``
    steps (``netket/_src/callbacks/observables.py:8-48``)."""

    def __init__(self, observables, interval=1):
        self._observables = {} if observables is None else observables
        self._interval = interval
        self._last_step = float("-inf")

    def before_parameter_update(self, step, log_data, driver):
        if step >= self._last_step + self._interval:
            log_data.update(driver.estimate(self._observables))
            self._last_step = step


class ProgressBarCallback(AbstractCallback):
    """A tqdm progress bar over the run's steps, showing the loss; nothing
    when tqdm is not installed."""

    def __init__(self, n_iter):
        self.n_iter = n_iter
        self._pbar = None

    def on_run_start(self, step, driver):
        try:
            from tqdm.auto import tqdm
        except ImportError:
            return
        self._pbar = tqdm(total=self.n_iter, dynamic_ncols=True)

    def on_step_end(self, step, log_data, driver):
        if self._pbar is None:
            return
        loss = log_data.get(driver._loss_name)
        if loss is not None:
            self._pbar.set_postfix_str(f"{driver._loss_name}={loss}")
        self._pbar.update(1)

    def _close(self):
        if self._pbar is not None:
            self._pbar.close()
            self._pbar = None

    def on_run_end(self, step, driver):
        self._close()

    def on_run_error(self, step, error, driver):
        self._close()


def _monitored(stats, monitor):
    return float(np.real(getattr(stats, monitor)))


class EarlyStopping(AbstractCallback):
    """Stops when the monitored loss statistic has not improved by
    ``min_delta`` (absolute) or ``min_reldelta`` (relative) for more than
    ``patience`` steps, or has not gone below ``baseline``
    (``netket/_src/callbacks/early_stopping.py``)."""

    def __init__(self, min_delta=0.0, min_reldelta=0.0, patience=0, baseline=None,
                 start_from_step=0, monitor="mean"):
        self.min_delta, self.min_reldelta = min_delta, min_reldelta
        self.patience, self.baseline = patience, baseline
        self.start_from_step, self.monitor = start_from_step, monitor
        self._best_val, self._best_iter, self._best_patience_counter = np.inf, 0, 0

    def _is_improvement(self, loss, target):
        return loss < min(target - self.min_delta, target * (1 - self.min_reldelta))

    def on_step_end(self, step, log_data, driver):
        if step < self.start_from_step:
            return
        loss = _monitored(log_data[driver._loss_name], self.monitor)
        self._best_patience_counter += 1
        if self._is_improvement(loss, self._best_val):
            self._best_val, self._best_iter = loss, step
            if self.baseline is None or self._is_improvement(loss, self.baseline):
                self._best_patience_counter = 0
        if self._best_patience_counter > self.patience:
            raise StopRun(f"EarlyStopping: no improvement detected after "
                          f"{self._best_patience_counter} steps (best value {self._best_val} "
                          f"at step {self._best_iter}).")


class InvalidLossStopping(AbstractCallback):
    """Stops once the monitored loss statistic has been non-finite for
    ``patience`` steps (``netket/_src/callbacks/invalid_loss_stopping.py``)."""

    def __init__(self, monitor="mean", patience=0):
        self.monitor, self.patience = monitor, patience
        self._last_valid_iter = 0

    def on_step_end(self, step, log_data, driver):
        if driver.step_count < self._last_valid_iter:
            self._last_valid_iter = 0
        if driver._loss_stats is None:
            return
        loss = _monitored(driver._loss_stats, self.monitor)
        if not np.isfinite(loss):
            if driver.step_count - self._last_valid_iter >= self.patience:
                raise StopRun(f"InvalidLossStopping: loss is not finite ({loss}) for "
                              f"{driver.step_count - self._last_valid_iter} steps.")
        else:
            self._last_valid_iter = driver.step_count


class Timeout(AbstractCallback):
    """Stops the run ``timeout`` seconds after it started
    (``netket/_src/callbacks/timeout.py``)."""

    def __init__(self, timeout):
        if not timeout > 0:
            raise ValueError("`timeout` must be larger than 0.")
        self.timeout = timeout
        self._init_time = None

    def on_run_start(self, step, driver):
        self._init_time = time.time()

    def on_step_end(self, step, log_data, driver):
        if time.time() - self._init_time >= self.timeout:
            raise StopRun(f"Timeout: training stopped after {self.timeout:.1f} seconds.")


class ConvergenceStopping(AbstractCallback):
    """Stops once the monitored loss statistic, averaged over the last
    ``smoothing_window`` steps, has been at or below ``target`` for more than
    ``patience`` consecutive steps
    (``netket/_src/callbacks/convergence_stopping.py``)."""

    def __init__(self, target, monitor="mean", *, smoothing_window=10, patience=10):
        self.target, self.monitor = target, monitor
        self.smoothing_window, self.patience = smoothing_window, patience
        self._loss_window = deque([], maxlen=smoothing_window)
        self._patience_counter = 0

    def on_step_end(self, step, log_data, driver):
        self._loss_window.append(_monitored(log_data[driver._loss_name], self.monitor))
        smooth = float(np.mean(self._loss_window))
        self._patience_counter = self._patience_counter + 1 if smooth <= self.target else 0
        if self._patience_counter > self.patience:
            raise StopRun(f"ConvergenceStopping: smoothed loss {smooth:.6g} has been below "
                          f"target {self.target} for {self._patience_counter} steps.")
