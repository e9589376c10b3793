"""Drivers (``netket.driver``): ``VMC`` and ``VMC_SR``.

The run loop mirrors ``netket/_src/driver/abstract_variational_driver.py:349-478``
(callbacks around computing the loss and update, step rejection, logging,
applying the optimiser; ``StopRun`` ends a run normally);
``VMC.compute_loss_and_update`` is ``netket/driver/vmc.py:141-158`` and
``VMC_SR.compute_loss_and_update`` is ``netket/_src/driver/vmc_sr.py:438-510``.
One step reads back exactly one small device buffer (the energy statistics and
the solver status); ``run`` adds the sampler's acceptance, as NetKet logs it.
"""
import numbers
import sys
import time
import warnings
from pathlib import Path

import torch

from . import callbacks as cb
from ._native import DEV_NO_CONVERGE, DEV_NONFINITE, DEV_NOT_SPD, DEV_TIMEOUT, VmckError
from .logging import JsonLog, RuntimeLog
from .ngd import minsr_fallback, minsr_update, sr_update
from .optimizer import identity_preconditioner
from .stats import Stats


class PhaseTimer:
    """CUDA events recorded between the phases of a step on the current stream
    (no host synchronisation); ``summary()`` syncs once and returns the mean
    milliseconds per phase.  The GPU counterpart of NetKet's ``timeit``
    (``netket/utils/timing.py``)."""

    def __init__(self):
        self.steps = []
        self._cur = None

    def mark(self, name):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        if name == "start":
            self._cur = [("start", ev)]
            self.steps.append(self._cur)
        elif self._cur is not None:
            self._cur.append((name, ev))

    def summary(self):
        torch.cuda.synchronize()
        acc = {}
        for marks in self.steps:
            for (_, a), (name, b) in zip(marks[:-1], marks[1:]):
                acc.setdefault(name, []).append(a.elapsed_time(b))
        return {k: sum(v) / len(v) for k, v in acc.items()}

    def reset(self):
        self.steps = []
        self._cur = None


class AbstractVariationalDriver:
    def __init__(self, variational_state, optimizer, minimized_quantity_name="Energy"):
        self.state = variational_state
        self.optimizer = optimizer
        self._loss_name = minimized_quantity_name
        self._loss_stats = None
        self._dp = None
        self.step_count = 0
        self.info = None
        self.phase_timer = None

    def compute_loss_and_update(self):
        raise NotImplementedError

    def reset(self):
        self.step_count = 0
        self.state.reset()

    def reset_step(self):
        self.state.reset()

    def update_parameters(self, dp):
        self.optimizer.apply(self.state, dp, self.step_count)

    def _accept_step(self):
        return True

    def advance(self, steps=1):
        for _ in range(steps):
            self._loss_stats, self._dp = self.compute_loss_and_update()
            self.update_parameters(self._dp)
            self.step_count += 1
        return self._loss_stats

    def iter(self, n_steps, step=1):
        for _ in range(0, n_steps, step):
            self.advance(step)
            yield self.step_count

    def estimate(self, observables):
        """``state.expect`` of an operator, or of each operator in a dict /
        list / tuple, in the same structure."""
        if isinstance(observables, dict):
            return {k: self.estimate(v) for k, v in observables.items()}
        if isinstance(observables, (list, tuple)):
            return type(observables)(self.estimate(v) for v in observables)
        return self.state.expect(observables)

    def _log_additional_data(self, log_dict):
        acc = getattr(getattr(self.state, "sampler_state", None), "acceptance", None)
        if acc is not None:
            log_dict["acceptance"] = acc
        log_dict["wallclock"] = time.perf_counter()

    def _default_callbacks(self, callbacks, n_iter, obs, step_size, loggers, show_progress):
        lst = [cb.maybe_wrap_legacy_callback(c) for c in callbacks]
        if obs is not None:
            lst.append(cb.ObservableCallback(obs, step_size))
        for lg in loggers:
            lst.append(lg if isinstance(lg, cb.AbstractCallback) else cb.LegacyLoggerWrapper(lg))
        if show_progress:
            lst.append(cb.ProgressBarCallback(n_iter))
        return cb.CallbackList(lst)

    def run(self, n_iter, out=(), obs=None, step_size=1, show_progress=True,
            save_params_every=50, write_every=50, callback=None, timeit=False):
        """Run ``n_iter`` steps (``abstract_variational_driver.py:349-478``).

        ``out``: a logger, an iterable of loggers, or a path prefix for a
        ``JsonLog`` (``save_params_every`` / ``write_every`` apply to it).
        ``obs``: operators estimated every ``step_size`` steps and logged beside
        the loss.  ``callback``: a function ``f(step, log_data, driver)`` (a falsy
        return stops the run) or an ``AbstractCallback``, or a list of them.
        ``timeit``: CUDA-event times of the step's phases, printed at the end
        and kept in ``self._timer``.  Returns the loggers."""
        if not isinstance(n_iter, numbers.Number):
            raise ValueError("n_iter, the first positional argument to `run`, must be a number!")
        if isinstance(out, (str, Path)):
            out = (JsonLog(out, "w", save_params_every, write_every),)
        elif out is None:
            out = ()
        loggers = tuple(out) if isinstance(out, (list, tuple)) else (out,)
        if callback is None:
            callback = ()
        elif not isinstance(callback, (list, tuple)):
            callback = (callback,)
        callbacks = self._default_callbacks(callback, n_iter, obs, step_size, loggers,
                                            show_progress)
        if timeit:
            self.phase_timer = PhaseTimer()
        t0 = time.perf_counter()
        try:
            callbacks.on_run_start(self.step_count, self)
            for _ in range(int(n_iter)):
                self._step_attempt = 0
                log_data = {}
                while True:
                    callbacks.on_step_start(self.step_count, log_data, self)
                    self.reset_step()
                    callbacks.on_compute_update_start(self.step_count, log_data, self)
                    self._loss_stats, self._dp = self.compute_loss_and_update()
                    reject = callbacks.on_compute_update_end(self.step_count, log_data, self)
                    if reject or not self._accept_step():
                        self._step_attempt += 1
                        continue
                    break
                if self._loss_stats is not None:
                    log_data[self._loss_name] = self._loss_stats
                self._log_additional_data(log_data)
                callbacks.before_parameter_update(self.step_count, log_data, self)
                self.update_parameters(self._dp)
                callbacks.on_step_end(self.step_count, log_data, self)
                self.step_count += 1
            callbacks.on_run_end(self.step_count, self)
        except cb.StopRun as error:
            callbacks.on_run_end(self.step_count, self)
            print(f"run stopped before the last step: {error}")
        except KeyboardInterrupt as error:
            callbacks.on_run_error(self.step_count, error, self)
            if hasattr(sys, "ps1"):
                print("Stopped by user.")
            else:
                raise
        except Exception as error:
            callbacks.on_run_error(self.step_count, error, self)
            raise
        finally:
            self.wall_time = time.perf_counter() - t0
            if timeit:
                self._timer = self.phase_timer.summary()
                self.phase_timer = None
                print({k: round(v, 3) for k, v in self._timer.items()})
        return loggers

    @property
    def energy(self):
        return self._loss_stats


class VMC(AbstractVariationalDriver):
    """``expect_and_grad`` then an optional preconditioner (e.g. ``SR``)."""

    def __init__(self, hamiltonian, optimizer, *, variational_state, preconditioner=None):
        if variational_state.hilbert != hamiltonian.hilbert:
            # netket/driver/vmc.py:77-84
            raise TypeError(f"the variational_state has hilbert space "
                            f"{variational_state.hilbert} (this is normally defined by the "
                            f"hilbert space in the sampler), but the hamiltonian has hilbert "
                            f"space {hamiltonian.hilbert}. The two should match.")
        super().__init__(variational_state, optimizer)
        self._ham = hamiltonian
        self.preconditioner = preconditioner or identity_preconditioner

    def compute_loss_and_update(self):
        self.state.reset()
        stats, grad = self.state.expect_and_grad(self._ham)
        dp = self.preconditioner(self.state, self.state.model.flatten(grad), self.step_count)
        return stats, dp


class VMC_SR(AbstractVariationalDriver):
    """Natural-gradient VMC: minSR (``use_ntk=True``) or SR, optionally SPRING
    (``momentum``, ``proj_reg``; ``netket/_src/driver/vmc_sr.py:146-176``).
    ``diag_shift``, ``proj_reg`` and ``momentum`` may be schedules
    ``step -> value``.

    ``use_ntk=None`` picks minSR when n_parameters > n_samples
    (``vmc_sr.py:356-357``).  ``gram``/``solve``/``gram_mode`` select the
    implementation of the minSR linear algebra (see ``netket_gb300.ngd``).
    """

    def __init__(self, hamiltonian, optimizer, *, diag_shift, variational_state, use_ntk=None,
                 gram="structured", gram_mode=None, solve=None, refine_iters=4,
                 refine_tol=1e-8, jac_dtype=None, proj_reg=None, momentum=None,
                 linear_solver=None, linear_solver_fn=None, chunk_size_bwd=None, mode=None,
                 on_the_fly=None):
        # linear_solver: NetKet's cholesky_with_fallback (default), cholesky (no
        # fallback) or pinv_smooth (netket/optimizer/solver/solvers.py); chunk_size_bwd
        # has no effect (nothing is chunked: the Jacobian is never materialised);
        # on_the_fly selects NetKet's srt_onthefly / srt, which here are one path.
        from .optimizer import solver as _solvers
        if linear_solver_fn is not None:
            # the reference's deprecated name for linear_solver (vmc_sr.py:264-266)
            if linear_solver is not None:
                raise ValueError("pass linear_solver only (linear_solver_fn is its deprecated "
                                 "name)")
            warnings.warn("linear_solver_fn is deprecated; use linear_solver",
                          FutureWarning, stacklevel=2)
            linear_solver = linear_solver_fn
        if linear_solver is None or linear_solver is _solvers.cholesky_with_fallback:
            self._solver = "fallback"
        elif linear_solver is _solvers.cholesky:
            self._solver = "cholesky"
        elif linear_solver is _solvers.pinv_smooth:
            self._solver = "pinv_smooth"
        else:
            raise NotImplementedError("VMC_SR: linear_solver must be one of "
                                      "optimizer.solver.cholesky_with_fallback / cholesky / "
                                      "pinv_smooth")
        if mode not in (None, "real"):
            raise NotImplementedError(f"VMC_SR: mode={mode!r}; the RBM path is real")
        if on_the_fly and use_ntk is False:
            raise NotImplementedError("on_the_fly SR (use_ntk=False) is not implemented")
        self.chunk_size_bwd = chunk_size_bwd
        self.on_the_fly = on_the_fly
        super().__init__(variational_state, optimizer)
        self.proj_reg = proj_reg
        self.momentum = momentum
        self._old_updates = None
        self._ham = hamiltonian
        self.diag_shift = diag_shift
        if use_ntk is None:
            use_ntk = variational_state.n_parameters > variational_state.n_samples
        self.use_ntk = bool(use_ntk)
        self.gram = gram
        self.gram_mode = gram_mode
        if solve is None:
            solve = "refined" if variational_state.precision == "mixed" else "cholesky"
        self.solve = solve
        self.refine_iters = refine_iters
        self.refine_tol = refine_tol
        self.jac_dtype = jac_dtype

    def compute_loss_and_update(self):
        st = self.state
        ph = self.phase_timer
        st.reset()
        if ph:
            ph.mark("start")
        st.sample()
        if ph:
            ph.mark("sample")
        c = st._forward_cache(self._ham)
        if ph:
            ph.mark("local_energy")
        step = self.step_count
        shift = self.diag_shift(step) if callable(self.diag_shift) else self.diag_shift
        proj_reg = self.proj_reg(step) if callable(self.proj_reg) else self.proj_reg
        mom = self.momentum(step) if callable(self.momentum) else self.momentum
        if mom is not None and self._old_updates is None:
            self._old_updates = torch.zeros(st.n_parameters, dtype=torch.float64,
                                            device=c["e"].device)
        old = self._old_updates if mom is not None else None
        if self.use_ntk:
            dp, self.info = minsr_update(c["t"], c["x"], st.N, st.M, c["e"], c["stats_dev"][0:1],
                                         shift, gram=self.gram, gram_mode=self.gram_mode,
                                         solve=self.solve, refine_iters=self.refine_iters,
                                         refine_tol=self.refine_tol, jac_dtype=self.jac_dtype,
                                         check=False, phase_timer=ph, proj_reg=proj_reg,
                                         momentum=mom, old_updates=old)
            # one host read per step: energy statistics and solver status together
            host = torch.cat([c["stats_dev"], self.info["status_dev"].to(torch.float64)]).cpu()
            status = int(host[5].item())
            self.info["status"] = status
            if status & DEV_TIMEOUT:
                raise VmckError("a device-side wait timed out in the minSR step")
            bad = DEV_NOT_SPD | DEV_NONFINITE
            if self.solve == "cholesky":
                bad |= DEV_NO_CONVERGE  # the FP64 solve's refinement did not converge
            failed = bool(status & bad)
            if self._solver == "pinv_smooth":
                dp = minsr_fallback(self.info, try_pcg=False)
            elif failed:
                # the FP32 factor failed: the FP64 solution by shifted-factor PCG,
                # else pinv_smooth (fallback) or NaN (a failed cho_factor)
                fb = minsr_fallback(self.info, pinv=self._solver == "fallback")
                dp = fb if fb is not None else torch.full_like(dp, float("nan"))
            stats = Stats.from_array(host[:5].numpy())
            if mom is not None:
                dp = dp + mom * old  # SPRING (netket/_src/ngd/srt.py:79-82)
        else:
            if proj_reg is not None:
                raise ValueError("proj_reg not implemented for SR")
            if self._solver != "fallback":
                raise NotImplementedError("VMC_SR(use_ntk=False) uses cholesky_with_fallback")
            dp, self.info = sr_update(c["t"], c["x"], st.N, st.M, c["e"], c["stats_dev"][0:1],
                                      shift, jac_dtype=self.jac_dtype, momentum=mom,
                                      old_updates=old)
            stats = Stats.from_array(c["stats_dev"].cpu().numpy())
        if mom is not None:
            self._old_updates = dp
        return stats, dp
