// Minimal, from-scratch stand-in for the parts of the ASL library (aslze/asl
// 1.11.14) that minirender's Renderer.cpp, Scene.cpp and primitives.cpp use.
// ASL itself is not available here; this header restates the behaviour of its
// public API only, so the reference sources compile unmodified into the oracle.
// Test infrastructure: never linked into the product library.
#ifndef ASL_SHIM_DEFS_H
#define ASL_SHIM_DEFS_H
#include <math.h>   // brings the float overloads (powf, floorf, tanf...) into scope
#include <stdlib.h>
#include <stdio.h>
#include <limits>
#include <utility>

namespace asl {

typedef unsigned char byte;

static const double PI = 3.14159265358979323846;
static const float PIf = 3.14159265f;

inline float infinity() { return std::numeric_limits<float>::infinity(); }

// Scalar helpers.  Operation order is part of the restated contract:
// min/max pick `a` unless `b` is strictly smaller/larger; clamp tests the
// lower bound first.
template <class T> inline T min(T a, T b) { return (b < a) ? b : a; }
template <class T> inline T max(T a, T b) { return (a < b) ? b : a; }
template <class T> inline T clamp(T x, T lo, T hi) { return (x < lo) ? lo : ((x > hi) ? hi : x); }
inline float fract(float x) { return x - floorf(x); }
inline double fract(double x) { return x - floor(x); }
template <class T> inline void swap(T& a, T& b) { T t = a; a = b; b = t; }
inline float deg2rad(float d) { return d * (PIf / 180.0f); }

}  // namespace asl
#endif
