"""galario_gb300.double: drop-in for galario.double (float64 arrays, FP64 arithmetic on the GPU)."""
from ._module import make as _make

globals().update(_make("double"))
del _make
