// Scalar aliases of the reference (modules/include/cuda/types.cuh:7-22).
#ifndef CUPHOTO_GB300_TYPES_CUH
#define CUPHOTO_GB300_TYPES_CUH

#include <stdint.h>

namespace cuphoto {

using i8 = int8_t;
using ui8 = uint8_t;
using byte = i8;
using i16 = int16_t;
using ui16 = uint16_t;
using i32 = int32_t;
using i64 = int64_t;
using ui32 = uint32_t;
using ui64 = uint64_t;
using ul = unsigned long;
using r32 = float;
using r64 = double;
using sh16 = short;
using ush16 = unsigned short;
using ch = char;
using uch = unsigned char;

}  // namespace cuphoto

#endif
