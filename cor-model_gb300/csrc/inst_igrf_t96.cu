// Kernels of the model set {internal 1, external 1, crustal 0}.
#include "inst.cuh"

COR_MODEL_INSTANCE(igrf_t96, 1, 1, 0)
