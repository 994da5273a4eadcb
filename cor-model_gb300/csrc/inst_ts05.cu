// Kernels of the model set {internal 0, external 2, crustal 0}.
#include "inst.cuh"

COR_MODEL_INSTANCE(ts05, 0, 2, 0)
