/* On hosts without x86 intrinsics (the aarch64 GPU hosts), the reference's
 * #include "immintrin.h" (include/Physecs/SIMD.h:3) resolves here: the SSE
 * subset the reference uses, emulated lane by lane with the same IEEE
 * single-precision operations.  Test infrastructure only. */
#pragma once
#include "../psx_sse_portable.h"
