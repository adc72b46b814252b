"""GB300-native symmetry hot path (curvature, pair voting, mean-shift,
verification) behind the reference's Backend interface.

The compute runs in hand-written sm_103a kernels in ``_lib/libmitra_gb300.so``
reached through the C ABI of include/mitra_gb300.h.
"""
from .types import (ClusterOutput, Csr, Features, Mesh, ModelContext, Options, Pairs, Rng,
                    Selection, Topology, Verification, Votes)

__all__ = ["ClusterOutput", "Csr", "Features", "Mesh", "ModelContext", "Options", "Pairs", "Rng",
           "Selection", "Topology", "Verification", "Votes", "Gb300Backend", "detect"]


def __getattr__(name):
    if name in ("Gb300Backend", "detect"):
        from . import backend
        return getattr(backend, name)
    raise AttributeError(name)
