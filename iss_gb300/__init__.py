"""GB300-native Cooper-Frye hadron sampler (the FSSW path of iSS).

    from iss_gb300 import iSS
    s = iSS(path, inputfile="iSS_parameters.dat")
    s.shell()                       # read surface, seed, sample on the GPU
    hadrons, event_offsets = s.all_hadrons()

The compute path is the native library built from iss_gb300/csrc (C ABI in
include/iss_gpu.h, CUDA kernels for sm_103a)."""
from .native import (HADRON_DTYPE, OUTPUT_BINARY, OUTPUT_GZIP, OUTPUT_OSCAR, TABLE_DIR,  # noqa: F401
                     IssError, iSS, lib)

__all__ = ["iSS", "IssError", "lib", "HADRON_DTYPE", "TABLE_DIR", "OUTPUT_OSCAR",
           "OUTPUT_GZIP", "OUTPUT_BINARY"]
