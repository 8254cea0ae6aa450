"""piqmc on GB300: path-integral quantum annealing with the reference's Python API.

Drop-in modules: ``piqmc.qmc`` (QuantumAnneal, QuantumAnneal_dense), ``piqmc.sa``
(Anneal, ClassicalIsingEnergy), ``piqmc.tools`` (GenerateNeighbors,
bits2spins, spins2bits).  Batched device-level APIs: ``piqmc.fast`` (packed
sweeps over many replicas) and ``piqmc.reforder`` (reference-order sweeps with
explicit streams).  All compute runs in ``libpiqmc_gb300.so`` on a CUDA device.
"""
from . import _native  # noqa: F401

__all__ = ["qmc", "sa", "tools", "fast", "reforder"]
__version__ = "0.1.0"


def __getattr__(name):
    if name in __all__:
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
