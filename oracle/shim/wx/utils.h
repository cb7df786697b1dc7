// Test-infrastructure shim (oracle only). wxLongLong as a 64-bit integer
// wrapper, free memory and disk queries, and wxSetWorkingDirectory. The oracle
// always runs in-core: the free-memory query reports a large figure.
#ifndef FCG_SHIM_WX_UTILS_H
#define FCG_SHIM_WX_UTILS_H

#include <unistd.h>
#include "string.h"

class wxLongLong {
public:
    long long v;
    wxLongLong() : v(0) {}
    wxLongLong(long long x) : v(x) {}
    long ToLong() const { return (long)v; }
    double ToDouble() const { return (double)v; }
    void Assign(double d) { v = (long long)d; }
};
inline wxLongLong operator*(const wxLongLong &a, const wxLongLong &b) { return wxLongLong(a.v * b.v); }
inline wxLongLong operator/(const wxLongLong &a, const wxLongLong &b) { return wxLongLong(a.v / b.v); }
inline wxLongLong operator%(const wxLongLong &a, const wxLongLong &b) { return wxLongLong(a.v % b.v); }
inline wxLongLong operator+(const wxLongLong &a, const wxLongLong &b) { return wxLongLong(a.v + b.v); }
inline wxLongLong operator-(const wxLongLong &a, const wxLongLong &b) { return wxLongLong(a.v - b.v); }
inline bool operator<(const wxLongLong &a, const wxLongLong &b) { return a.v < b.v; }
inline bool operator!=(const wxLongLong &a, const wxLongLong &b) { return a.v != b.v; }
inline bool operator==(const wxLongLong &a, const wxLongLong &b) { return a.v == b.v; }

typedef long long wxMemorySize;
inline wxMemorySize wxGetFreeMemory() { return (wxMemorySize)1 << 50; }
inline bool wxGetDiskSpace(const wxString &, wxLongLong *freeBytes) { if (freeBytes) *freeBytes = wxLongLong((long long)1 << 50); return true; }
inline bool wxSetWorkingDirectory(const wxString &dir) { return dir.empty() || chdir(dir.c_str()) == 0; }

#endif
