"""GB300-native explicit MPM time step for Karamelo (TLMPM/ULMPM, USL/MUSL).

The hot path is hand-written sm_103a CUDA in ``csrc/`` behind the C ABI of
``include/kmpm.h``; :mod:`karamelo_gb300.model` mirrors Karamelo's
input-script commands on the host and :mod:`karamelo_gb300.gpu` drives the
library.
"""
from .model import MPM, KarameloError, TimeFn  # noqa: F401
