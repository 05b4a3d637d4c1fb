"""splatlight_gb300: Splatlight's per-frame splat pipeline (project -> stable depth sort -> per-tile ranges ->
front-to-back composite, with the per-Gaussian lighting it composites) as hand-written CUDA for GB300 (sm_103a),
behind a C ABI (include/splatlight.h, libsplatlight.so) with a Python host mirror of the reference's
SplatRenderer / Lighting objects."""
from .structs import FRAME, GAUSSIAN, MATERIAL, NODE, PART, VGRID  # noqa: F401

__version__ = "0.1.0"
