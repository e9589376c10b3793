"""netket_gb300: NetKet's VMC hot loop (Metropolis sampling, RBM amplitudes,
local energies, Jacobian contractions and the SR/minSR solve) as hand-written
sm_103a CUDA kernels behind a C ABI (``include/vmck.h``, ``libvmck.so``), with a
host API that mirrors ``netket``: ``hilbert``, ``graph``, ``operator``,
``models``, ``sampler``, ``vqs``, ``stats``, ``optimizer``, ``driver``,
``logging``, ``callbacks``, ``exact``, ``nn``.
"""
from . import _native
from . import graph
from . import hilbert
from . import operator
from . import nn
from . import models
from . import sampler
from . import stats
from . import kernels
from . import ngd
from . import optimizer
from . import vqs
from . import logging
from . import callbacks
from . import driver
from . import exact
from . import batched
from . import serving
from . import serialization

__all__ = ["graph", "hilbert", "operator", "models", "sampler", "stats", "kernels", "ngd", "batched", "serving", "serialization",
           "optimizer", "vqs", "driver", "logging", "callbacks", "exact", "nn"]
