"""galario_gb300: GB300-native synthetic visibilities and chi-squared for radio interferometry.

Drop-in for the reference package ``galario`` (v1.2.2, ``python/__init__.py.in``):

    import galario_gb300 as galario
    from galario_gb300 import double      # float64, as galario.double
    from galario_gb300 import single      # float32, as galario.single

``double_cuda`` and ``single_cuda`` are the same modules (everything runs on
the GPU; there is no CPU back end).
"""
from . import double, single
from ._module import arcsec, deg, cgs_to_Jy, pc, au

double_cuda = double
single_cuda = single
HAVE_CUDA = True
__version__ = "0.1.0"

__all__ = ["double", "single", "double_cuda", "single_cuda", "HAVE_CUDA",
           "arcsec", "deg", "cgs_to_Jy", "pc", "au"]
