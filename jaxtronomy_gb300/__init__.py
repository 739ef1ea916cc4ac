"""GB300-native lens image simulation with JAXtronomy's ImageModel / LensModel /
LightModel kwargs-list API.

All compute runs in ``liblensgb.so`` (hand-written sm_103a CUDA kernels behind a
C ABI, ``include/lensgb.h``); build it with ``python -m jaxtronomy_gb300.build``.
"""

from .data import ImageData, PSF, PixelGrid  # noqa: F401
from .image_model import ImageModel  # noqa: F401
from .lens_model import LensModel  # noqa: F401
from .cosmology import FlatLambdaCDM  # noqa: F401
from .lens_model_bulk import LensModelBulk, MultiPlaneBulk, SinglePlaneBulk  # noqa: F401
from .light_model import LightModel  # noqa: F401
from .point_source import PointSource  # noqa: F401
from .sampling import ImageLikelihood, LikelihoodModule, Param, prepare_logL_func  # noqa: F401

__version__ = "0.1.0"

__all__ = ["ImageData", "PSF", "PixelGrid", "ImageModel", "LensModel", "LensModelBulk", "LightModel",
           "MultiPlaneBulk", "SinglePlaneBulk", "FlatLambdaCDM", "PointSource",
           "ImageLikelihood", "LikelihoodModule", "Param", "prepare_logL_func"]
