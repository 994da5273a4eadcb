// Kernels of the model set {internal 1, external 2, crustal 0}.
#include "inst.cuh"

COR_MODEL_INSTANCE(igrf_ts05, 1, 2, 0)
