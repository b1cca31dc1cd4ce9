"""GB300-native image-based-lighting precompute (irradiance, GGX prefilter
chain, split-sum BRDF LUT) behind a C ABI (include/althea_ibl.h)."""
from . import ibl, synth  # noqa: F401
from .ibl import IBLHandles, IBLResources, ImageBasedLighting  # noqa: F401
