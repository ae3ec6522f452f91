/* Forced-include prelude for compiling the reference sources with g++.
 *  - MSVC names (fopen_s, _isnan, _finite, sscanf_s) mapped to POSIX/C++.
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
#define sscanf_s sscanf
