// Kernels of the model set {internal 1, external 0, crustal 0}.
#include "inst.cuh"

COR_MODEL_INSTANCE(igrf, 1, 0, 0)
