// Replacement for the reference's include/memory_copy.cuh in the
// reference-build harness, found first on the include path.
//
// The reference header only compiles under MSVC (an extra `MemoryCopy::`
// qualification inside the class and `static` on out-of-class member
// template definitions, memory_copy.cuh:27-49).  Of that header the
// reference's sources use only the two __constant__ symbols and
// MemoryCopy::copyConstant() (memory_copy.cu:5-12, calculation.cu:16); this
// file declares exactly those, with the same names and types.
#ifndef _MEMCOPY_CUH
#define _MEMCOPY_CUH

#include "cuda_macro.cuh"
#include "function.cuh"
#include "sim.cuh"

#include "cuda_runtime.h"

extern __constant__ Parameter dev_par;
extern __constant__ Data_Pointer dev_data;

class MemoryCopy : public DeviceFunction
{
public:
    static void copyConstant();
};

#endif
