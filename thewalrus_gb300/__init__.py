"""thewalrus_gb300: the hafnian / loop-hafnian finite-difference sieve of The Walrus on GB300.

Drop-in replacements for ``thewalrus.hafnian``, ``hafnian_repeated``, ``loop_hafnian`` and
``thewalrus.loop_hafnian_batch.loop_hafnian_batch`` and
``thewalrus.loop_hafnian_batch_gamma.loop_hafnian_batch_gamma`` backed by hand-written sm_103a CUDA kernels
(``csrc/``) behind a C ABI (``include/walrus_gb300.h``).
"""
from ._hafnian import (
    hafnian,
    hafnian_repeated,
    loop_hafnian,
    loop_hafnian_batch,
    loop_hafnian_batch_gamma,
    hafnian_batch,
    input_validation,
    reduction,
    matched_reps,
    prepare_hafnian,
    prepare_loop_hafnian,
    prepare_loop_hafnian_batch,
    prepare_loop_hafnian_batch_gamma,
    hafnian_with_error,
    run_with_magnitudes,
)
from . import _native as native

__version__ = "0.1.0"

__all__ = [
    "hafnian",
    "hafnian_repeated",
    "loop_hafnian",
    "loop_hafnian_batch",
    "loop_hafnian_batch_gamma",
    "hafnian_batch",
    "input_validation",
    "reduction",
    "matched_reps",
    "prepare_hafnian",
    "prepare_loop_hafnian",
    "prepare_loop_hafnian_batch",
    "prepare_loop_hafnian_batch_gamma",
    "hafnian_with_error",
    "run_with_magnitudes",
    "native",
    "version",
]


def version():
    """Version string of this package."""
    return __version__
