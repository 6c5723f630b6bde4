"""GB300-native MUSCL-Hancock + constrained-transport MHD stage (drop-in for godunov_mhd_ct's
GodunovImplemV0 hot path)."""
from .mesh import BlockMesh  # noqa: F401
