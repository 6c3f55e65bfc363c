"""flare_pp_gb300: the flare++ prediction path (B2 / B3 descriptors, the
NormalizedDotProduct kernel against a sparse set, SparseGP mean / SOR
prediction and the mapped-beta pair style) on GB300 GPUs.

The compute runs in libflare_pp_gb300.so (C ABI in include/flare_pp_gb300.h);
this package is its Python face, mirroring the reference's _C_flare names.
"""
from .api import (B2, B3, ClusterDescriptor, ComputeFlareStdAtom, DescriptorValues,
                  NormalizedDotProduct, PairFLARE, SparseGP, Structure)

__all__ = ["B2", "B3", "ClusterDescriptor", "ComputeFlareStdAtom", "DescriptorValues",
           "NormalizedDotProduct", "PairFLARE", "SparseGP", "Structure"]
