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
struct CString {
    CString(const char* = 0) {}
    void Format(const char*, ...) {}
    CString& operator+=(const CString&) { return *this; }
    CString& operator+=(const char*) { return *this; }
};
struct _timeb { long long time; unsigned short millitm; };
static inline void _ftime_s(struct _timeb* t) { t->time = 0; t->millitm = 0; }
static inline int AfxMessageBox(const CString&) { return 0; }
struct CFile {};
struct CException { void Delete() {} };
struct CGazoApp {};
static inline void* AfxGetApp() { return 0; }
#endif
