"""Import the reference package (larsgeb/hmclab) in a container that lacks its
plotting / HDF5 / widget dependencies.

TEST INFRASTRUCTURE ONLY.  This module is used by the golden-fixture generator
(`tests/golden/make_golden.py`) to run the reference's own numpy code on seeded
inputs.  The product package never imports it, and it cannot run where the
reference sources are absent (it returns None from `load()` there).

Why the stubs are needed: `hmclab/__init__.py:4-10` imports `Samplers`, which
imports h5py, multiprocess, matplotlib, ipywidgets and IPython
(`hmclab/Samplers.py:33-53`); none of those are needed for the numpy HMC path when
the samples file ends in `.npy` (`hmclab/Samples.py:31-32,146-151`).
"""
import os
import sys
import types
from unittest import mock


def _reference_root():
    """The reference checkout: $HMCLAB_REFERENCE_ROOT when set, else a
    directory named `reference` beside this repository (absent on machines
    that only run the device tests, where load() returns None)."""
    env = os.environ.get("HMCLAB_REFERENCE_ROOT")
    if env:
        return env
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return os.path.join(os.path.dirname(repo), "reference")


REFERENCE_ROOT = _reference_root()

_STUBBED = [
    "h5py",
    "matplotlib",
    "matplotlib.pyplot",
    "matplotlib.gridspec",
    "matplotlib.colors",
    "matplotlib.cm",
    "matplotlib.ticker",
    "matplotlib.patches",
    "mpl_toolkits",
    "mpl_toolkits.axes_grid1",
    "mpl_toolkits.axes_grid1.axes_divider",
    "ipywidgets",
    "IPython",
    "IPython.display",
]


def load():
    """Return the imported `hmclab` reference package, or None if unavailable."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "hmclab")):
        return None
    for name in _STUBBED:
        if name not in sys.modules:
            sys.modules[name] = mock.MagicMock(name=name)
    if "multiprocess" not in sys.modules:
        import multiprocessing

        mp = types.ModuleType("multiprocess")
        for attr in ("Process", "Pipe", "Value", "Queue", "Pool", "cpu_count"):
            setattr(mp, attr, getattr(multiprocessing, attr))
        sys.modules["multiprocess"] = mp
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import hmclab  # noqa: F401
    return hmclab
