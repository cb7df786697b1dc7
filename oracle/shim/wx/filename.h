// Test-infrastructure shim (oracle only). The wxFileName members the
// reference calls to resolve the input path and name temporary files,
// restated with POSIX calls.
#ifndef FCG_SHIM_WX_FILENAME_H
#define FCG_SHIM_WX_FILENAME_H

#include <string>
#include <stdlib.h>
#include <unistd.h>
#include <limits.h>
#include "string.h"

class wxFileName {
public:
    wxString m_full;
    wxFileName() {}
    void Assign(const wxString &full) { m_full = full; }
    void Assign(const wxString &dir, const wxString &name) {
        m_full = dir;
        if (!m_full.empty() && m_full[m_full.size() - 1] != '/') m_full += "/";
        m_full += name;
    }
    void Clear() { m_full.clear(); }
    bool FileExists() const { return access(m_full.c_str(), F_OK) == 0; }
    bool IsOk() const { return !m_full.empty(); }
    bool MakeAbsolute() {
        if (!m_full.empty() && m_full[0] == '/') return true;
        char cwd[PATH_MAX];
        if (getcwd(cwd, sizeof(cwd)) == NULL) return false;
        m_full = wxString(cwd) + "/" + m_full;
        return true;
    }
    bool IsFileReadable() const { return access(m_full.c_str(), R_OK) == 0; }
    wxString GetFullPath() const { return m_full; }
    wxString GetLongPath() const { return m_full; }
    wxString GetPath() const {
        size_t p = m_full.rfind('/');
        return p == std::string::npos ? wxString("") : wxString(m_full.substr(0, p));
    }
    wxString GetFullName() const {
        size_t p = m_full.rfind('/');
        return p == std::string::npos ? m_full : wxString(m_full.substr(p + 1));
    }
    static wxString GetTempDir() { const char *t = getenv("TMPDIR"); return wxString(t ? t : "/tmp"); }
    static void SplitPath(const wxString &full, wxString *dir, wxString *name, wxString *ext) {
        size_t p = full.rfind('/');
        if (dir) *dir = p == std::string::npos ? wxString("") : wxString(full.substr(0, p));
        if (name) *name = p == std::string::npos ? full : wxString(full.substr(p + 1));
        if (ext) *ext = wxString("");
    }
};

#endif
