"""GB300-native (sm_103a) streaming hot path of streamParanumal: BS0-BS8.

The compute runs in ``lib/libspgb300.so`` (hand-written CUDA kernels behind the C
ABI of ``include/sp_capi.h``).  This package binds that ABI (:mod:`.capi`) and
mirrors the reference's kernel calls (:mod:`.kernels`) and ``ogs_t`` handle
(:mod:`.ogs`).
"""
from . import capi  # noqa: F401

__all__ = ["capi", "kernels", "ogs"]
__version__ = "0.1.0"


def __getattr__(name):
    if name in ("kernels", "ogs"):
        import importlib

        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
