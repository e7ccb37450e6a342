// Minimal stand-in for the reference's ctypes.h (whose __fp16 typedef does not
// compile on x86-64).  Declares the border and error enums with the reference's
// values (kleidicv/include/kleidicv/ctypes.h:26-79), nothing else.
#ifndef KCV_PROBE_STUB_CTYPES_H
#define KCV_PROBE_STUB_CTYPES_H
#include <cstddef>
#include <cstdint>
#include "kleidicv/config.h"
typedef enum {
  KLEIDICV_OK = 0,
  KLEIDICV_ERROR_NOT_IMPLEMENTED,
  KLEIDICV_ERROR_NULL_POINTER,
  KLEIDICV_ERROR_RANGE,
  KLEIDICV_ERROR_ALLOCATION,
  KLEIDICV_ERROR_ALIGNMENT,
  KLEIDICV_ERROR_CONTEXT_MISMATCH,
} kleidicv_error_t;
typedef enum {
  KLEIDICV_BORDER_TYPE_CONSTANT,
  KLEIDICV_BORDER_TYPE_REPLICATE,
  KLEIDICV_BORDER_TYPE_REFLECT,
  KLEIDICV_BORDER_TYPE_WRAP,
  KLEIDICV_BORDER_TYPE_REVERSE,
  KLEIDICV_BORDER_TYPE_TRANSPARENT,
  KLEIDICV_BORDER_TYPE_NONE,
} kleidicv_border_type_t;
#endif
