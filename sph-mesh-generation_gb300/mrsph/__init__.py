"""mrsph — GB300-native adaptive SPH particle relaxation (the data-parallel
core of the SPH mesh generator Xiangyu-Hu/SPH-mesh-generation) behind the C
ABI of include/mrsph_relax.h."""
from . import cases, io  # noqa: F401
from .solver import BatchRelaxation, SPHMeshGeneration  # noqa: F401

__all__ = ["cases", "io", "SPHMeshGeneration", "BatchRelaxation"]
