"""galario_gb300.single: drop-in for galario.single (float32 arrays; FP32 spectrum with FP64
uv-to-grid index, phase-argument reduction and chi2 accumulation)."""
from ._module import make as _make

globals().update(_make("single"))
del _make
