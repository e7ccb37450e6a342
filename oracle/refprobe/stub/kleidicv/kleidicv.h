// Minimal stand-in for the reference's kleidicv.h (AArch64-only).  The border
// tables include it only for the C types.
#ifndef KCV_PROBE_STUB_KLEIDICV_H
#define KCV_PROBE_STUB_KLEIDICV_H
#include "kleidicv/ctypes.h"
#endif
