"""GB300-native cochlear solver: BM/OHC adaptive-step solver, IHC/lambda
filters and JND, behind the C ABI of include/cochlea_gb300.h."""
from . import native  # noqa: F401
from .model import ModelVectors, RunConfig, bm_scalars, reference_units  # noqa: F401

__all__ = ["native", "ModelVectors", "RunConfig", "bm_scalars", "reference_units"]
