"""coldcase_gb300 -- GB300 (sm_103a) covering-code search and verification.

The covering-code hot path of Mapika/coldcase rebuilt for one GB300: the
sphere-walk tabu engine of cov/engine/covsearch2e.c (bit-identical
trajectory) and the distance transform / coverage count behind
cov/verify_cov.py, as hand-written CUDA behind the C ABI of
include/covgpu.h (libcovgpu.so), with Python host code on top.
"""
from . import codefile  # noqa: F401
from .lib import CovError, load  # noqa: F401

__all__ = ["codefile", "CovError", "load", "engine", "verify"]


def __getattr__(name):
    if name in ("engine", "verify", "batch", "serve"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
