"""Launch-shape autotuner of the CUDA library (C ABI ``tprf_set_autotune``,
``tprf_autotune_*``), in the spirit of FFTW's planner: ``set_autotune(True)``
makes the first call of each shape time its candidate launch shapes and keep
the fastest; ``save_wisdom`` / ``load_wisdom`` carry the choices across
processes. Results do not depend on the mode, only the speed does.
"""
from __future__ import annotations

import contextlib
import os

from . import _native

__all__ = ["set_autotune", "autotune_enabled", "wisdom_entries", "clear_wisdom", "save_wisdom", "load_wisdom",
           "tuned"]


def set_autotune(on: bool = True) -> None:
    _native.check(_native.lib().tprf_set_autotune(1 if on else 0), "set_autotune")


def autotune_enabled() -> bool:
    return bool(_native.lib().tprf_get_autotune())


def wisdom_entries() -> int:
    return int(_native.lib().tprf_autotune_entries())


def clear_wisdom() -> None:
    _native.lib().tprf_autotune_clear()


def save_wisdom(path) -> None:
    _native.check(_native.lib().tprf_autotune_save(os.fsencode(path)), "autotune_save")


def load_wisdom(path) -> None:
    _native.check(_native.lib().tprf_autotune_load(os.fsencode(path)), "autotune_load")


@contextlib.contextmanager
def tuned(path=None, measure: bool = True):
    """The FFTW-style workflow in one block: the choices in ``path`` (when it
    exists) are loaded, measure mode is on inside the block (``measure``), and
    on leaving it the mode returns to what it was and every choice (loaded or
    newly measured) is written back to ``path``, so the next process starts
    from them and times nothing it has timed before. ``path=None`` keeps the
    choices in this process only."""
    was = autotune_enabled()
    if path is not None and os.path.exists(path):
        load_wisdom(path)
    set_autotune(measure)
    try:
        yield
    finally:
        set_autotune(was)
        if path is not None:
            save_wisdom(path)
