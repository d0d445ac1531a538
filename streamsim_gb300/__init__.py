"""GB300-native FacetRT facet radiosity (StreamSim HiStream eFacetRT path).

The compute lives in libfacetcu.so (CUDA, sm_103a) behind the C ABI of
include/facetcu.h; `facetcu` binds it with ctypes and mirrors the reference's
facetvk::FacetrtVulkan interface; `scenes` builds the synthetic workloads.
"""
from . import facetcu, scenes  # noqa: F401

__all__ = ["facetcu", "scenes"]
