// Test-infrastructure shim (oracle only). wxWidgets is not installed; this
// restates the few wxString members the reference's headless solver code uses
// (construction from C strings, (const char*) conversion, c_str(), +, +=,
// Clear(), Format()) on top of std::string, plus the wxT/_T macros.
#ifndef FCG_SHIM_WX_STRING_H
#define FCG_SHIM_WX_STRING_H

#include <string>
#include <stdarg.h>
#include <stdio.h>
#include <cstring>
#include <iostream>

#define wxT(x) x
#ifndef _T
#define _T(x) x
#endif
typedef char wxChar;

class wxString : public std::string {
public:
    wxString() {}
    wxString(const char *s) : std::string(s ? s : "") {}
    wxString(const std::string &s) : std::string(s) {}
    operator const char *() const { return c_str(); }
    void Clear() { clear(); }
    wxString &operator+=(const char *s) { append(s); return *this; }
    wxString &operator+=(const std::string &s) { append(s); return *this; }
    static wxString Format(const char *fmt, ...) {
        char buf[4096];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        return wxString(buf);
    }
};

inline wxString operator+(const wxString &a, const wxString &b) { return wxString(static_cast<const std::string &>(a) + static_cast<const std::string &>(b)); }
inline wxString operator+(const wxString &a, const char *b) { return wxString(static_cast<const std::string &>(a) + b); }
inline wxString operator+(const char *a, const wxString &b) { return wxString(a + static_cast<const std::string &>(b)); }

#endif
