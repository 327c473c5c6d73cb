"""photon_gb300: GB300-native (sm_103a) wavefront path tracer behind Photon's
renderer seam and ray back-end interface (see include/photon_cuda.h)."""
from . import _abi  # noqa: F401
from .native import PhotonError, load  # noqa: F401
from .renderer import Accel, Renderer, tuning_get, tuning_set  # noqa: F401
from .scene import SceneData, camera, settings  # noqa: F401
from .renderer import render_batch  # noqa: F401,E402
