// Test-infrastructure shim (oracle only): wxASSERT compiled out.
#ifndef FCG_SHIM_WX_DEBUG_H
#define FCG_SHIM_WX_DEBUG_H
#define wxASSERT(x) ((void)0)
#endif
