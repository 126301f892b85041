"""hmclab_gb300 — the Hamiltonian Monte Carlo hot path of hmclab on one GB300.

Drop-in modules with the reference's names (larsgeb/hmclab):
`Distributions`, `MassMatrices`, `Samplers`, `Samples`.  All arithmetic runs in
the in-tree CUDA library `libhmclab_gb300.so` (sm_103a); there is no CPU
fallback.
"""
from hmclab_gb300 import Distributions, MassMatrices, Samplers  # noqa: F401
from hmclab_gb300.Samples import Samples, combine_samples  # noqa: F401

__version__ = "0.1.0"
__all__ = ["Distributions", "MassMatrices", "Samplers", "Samples", "combine_samples"]
