/* Forced-include prelude for compiling the reference sources with g++.
 *  - MSVC names (fopen_s, _isnan, _finite, sscanf_s) mapped to POSIX/C++.
 *    sscanf_s keeps MSVC's argument convention (a buffer size after each
 *    string pointer), so the reference's .obj reader runs unchanged.
 *  - `using std::abs`: MSVC resolves the reference's unqualified abs(float)
 *    to the floating overload; without this g++ picks int abs() and every
 *    cosine term collapses (ray.cpp:55, camera.cpp:39, kdtree.cpp:203 ...).
 *  - std::powf / std::sqrtf / std::fabsf, which MSVC provides in std.     */
#pragma once
#include <cmath>
#include <math.h>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <climits>
#include <limits>
#include <string>
#include <iostream>
#include <algorithm>
using std::abs;
namespace std {
using ::powf;
using ::sqrtf;
using ::fabsf;
}
#define fopen_s(pf, name, mode) ((*(pf) = fopen((name), (mode))) ? 0 : 1)
#define _isnan(x) std::isnan(x)
#define _finite(x) std::isfinite(x)
#include <cstdarg>
/* MSVC's sscanf_s: after the pointer of each %s, %c or %[ conversion comes
 * that buffer's size (unsigned); other conversions take one pointer, and
 * surplus trailing arguments are ignored.  Collects the pointers in order and
 * calls sscanf with them (at most 16 conversions, which covers mesh.cpp and
 * config.cpp). */
static inline int wr_sscanf_s(const char* str, const char* fmt, ...) {
    void* p[16] = {0};
    int n = 0;
    va_list ap;
    va_start(ap, fmt);
    for (const char* f = fmt; *f && n < 16; f++) {
        if (*f != '%') continue;
        f++;
        if (*f == '%') continue;
        const bool skip = *f == '*';
        while (*f && !strchr("diouxXeEfgGaAcspn[", *f)) f++;  // width and length modifiers
        if (!*f) break;
        const char conv = *f;
        if (conv == '[')
            while (*f && *f != ']') f++;
        if (skip) continue;
        p[n++] = va_arg(ap, void*);
        if (conv == 's' || conv == 'c' || conv == '[') (void)va_arg(ap, unsigned);
    }
    va_end(ap);
    return sscanf(str, fmt, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[10], p[11], p[12],
                  p[13], p[14], p[15]);
}
#define sscanf_s wr_sscanf_s
