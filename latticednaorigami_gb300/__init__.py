"""GB300-native batched Monte Carlo engine for the lattice DNA-origami model
of cumberworth/LatticeDNAOrigami: hand-written sm_103a CUDA kernels behind a
C ABI (include/ldo.h), driven from the reference's own input files."""
from .engine import Batch, Engine, LdoError, Observables, load_library, LIB_PATH, EXPORTS  # noqa: F401
