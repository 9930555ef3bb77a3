// Stand-in for <cuComplex.h>: the reference's src/demag_cu.cu includes it but
// uses only the float2 / double2 types (declared in the cuda_runtime.h stand-in).
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include "cuda_runtime.h"
