// Kernels of every model set with the crustal model: the internal and
// external models are chosen at run time (CrustalTables::internal/external).
#include "inst.cuh"

COR_MODEL_INSTANCE(crustal, kModelAtRunTime, kModelAtRunTime, 1)
