"""CPU oracle for the VMC hot path (TEST INFRASTRUCTURE ONLY).

This package is a plain numpy/scipy FP64 restatement of NetKet's VMC hot loop.
It exists to check the CUDA path; it is never the thing that is measured or
shipped.  Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it.  The product package
``netket_gb300`` never imports it and fails loudly when its CUDA library is
missing.

Each function cites the NetKet file:line it restates (paths relative to the
NetKet source tree).  The restatement is pinned against golden vectors that
``tests/golden/make_golden.py`` produced by executing the reference's own
pure-Python / numba-kernel source in this container (numba replaced by a
pass-through decorator, jax.numpy by numpy where the code is array-only).

Modules:
  graph     lattice edges (Hypercube/Square/Chain), hop distances, bipartiteness
  hilbert   spin-1/2 encoding and random states
  operator  Ising and LocalOperator/Heisenberg get_conn_padded
  rbm       RBM log-amplitude, log_cosh, analytic Jacobian
  sampler   Metropolis Local/Exchange sweeps (numpy RNG; distributional parity)
  stats     blocking statistics estimator (mean, variance, error, tau, split R-hat)
  ngd       SR / minSR updates, Cholesky with pinv_smooth fallback, SGD
  exact     sparse Hamiltonian, Lanczos ground state, full-sum expectations
"""
