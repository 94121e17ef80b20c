/* Minimal stand-ins for the MFC/Win32 names that the reference's hot-path sources mention, so
 * that those sources compile unmodified on Linux inside the oracle's reference build.
 * TEST INFRASTRUCTURE ONLY (oracle/build_ref.sh). */
#ifndef RVREF_AFX_H_
#define RVREF_AFX_H_
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
typedef int BOOL;
typedef unsigned long DWORD;
typedef uintptr_t DWORD_PTR;
typedef unsigned int COLORREF;
typedef size_t rsize_t;
typedef const char* LPCTSTR;
#define TRUE 1
#define FALSE 0
#define __stdcall
#define __int64 long long
#include <stdarg.h>
#include <string>
#include <vector>
/* a small std::string-backed CString: the members the extracted functions use */
struct CString {
    std::string s;
    CString(const char* p = 0) : s(p ? p : "") {}
    void Format(const char* fmt, ...) {
        char buf[4096];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        s = buf;
    }
    int GetLength() const { return (int)s.size(); }
    CString Left(int n) const { return CString(s.substr(0, n < 0 ? 0 : (size_t)n).c_str()); }
    CString& operator+=(const CString& o) { s += o.s; return *this; }
    CString& operator+=(const char* o) { s += o; return *this; }
    operator const char*() const { return s.c_str(); }
};
template <size_t N> static inline int strcpy_s(char (&dst)[N], const char* src) {
    strncpy(dst, src, N - 1);
    dst[N - 1] = 0;
    return 0;
}
struct _timeb { long long time; unsigned short millitm; };
static inline void _ftime_s(struct _timeb* t) { t->time = 0; t->millitm = 0; }
static inline int AfxMessageBox(const CString&) { return 0; }
/* CFile that appends to a byte buffer (the TIFF writer's output) */
struct CFile {
    std::vector<unsigned char> bytes;
    void Write(const void* p, unsigned int n) {
        const unsigned char* c = (const unsigned char*)p;
        bytes.insert(bytes.end(), c, c + n);
    }
};
struct CException { void Delete() {} };
struct CGazoApp {};
static inline void* AfxGetApp() { return 0; }
#endif
