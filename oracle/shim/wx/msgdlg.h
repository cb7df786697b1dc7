// Test-infrastructure shim (oracle only): no dialogs in the headless oracle.
#ifndef FCG_SHIM_WX_MSGDLG_H
#define FCG_SHIM_WX_MSGDLG_H
#endif
