// Kernels of the model set {internal 0, external 1, crustal 0}.
#include "inst.cuh"

COR_MODEL_INSTANCE(t96, 0, 1, 0)
