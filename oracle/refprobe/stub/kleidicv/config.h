// Minimal stand-in for the reference's generated config.h, used only to
// include its header-only sigma generator and border tables on x86-64 for the
// oracle pinning probes.  Declares only the macros those headers use.
#ifndef KCV_PROBE_STUB_CONFIG_H
#define KCV_PROBE_STUB_CONFIG_H
#define KLEIDICV_TARGET_NAMESPACE kleidicv
#define KLEIDICV_STREAMING
#define KLEIDICV_API_DECLARATION(name, ...)
#endif
