/*
 * Force-included (g++ -include) into every translation unit of the reference
 * CPU build under oracle/_ref.  Test infrastructure only.
 *
 * It supplies what MSVC 2013 provided implicitly and g++ does not:
 *  - <cstdio>, <cstring>, <limits>, <cmath>, <cstdlib> (MSVC pulled these in
 *    transitively);
 *  - the float overloads of unqualified abs() at global scope, which MSVC's
 *    <cmath> declares; without them KinectFission/kifi/Mesher.cpp:143,153,163
 *    would bind abs(float) to the C int abs() under g++;
 *  - fopen_s / fprintf_s used by Mesher::Mesh2Obj (Mesher.cpp:58-73);
 *  - kifi::util::id<> for KinectFission/kifi/util/iterator.h:184, which MSVC
 *    resolved from a later include.
 */
#pragma once
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

using std::abs;

static inline int fopen_s(FILE** f, const char* name, const char* mode) {
    *f = std::fopen(name, mode);
    return *f ? 0 : errno;
}
#define fprintf_s std::fprintf

#include <kifi/util/functional.h>
