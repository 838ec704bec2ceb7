"""GB300-native collocation BEM (elastostatic / time-harmonic elastodynamic
quad8 SBIE assembly + dense LU) behind the C-ABI of include/mfbem.h, a drop-in
for MultiFEBE's build_lse_mechanics_bem_{staela,harela} and solve_lse_{r,c}."""
from . import meshgen, mshio
from ._abi import MfbemError, load as load_library
from .bem import BemRegion, LseState, solve_lse, sweep_harela_batch

__all__ = ["BemRegion", "LseState", "solve_lse", "sweep_harela_batch", "meshgen", "mshio", "MfbemError", "load_library"]
