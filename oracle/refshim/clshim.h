// Test infrastructure only (oracle): lets an OpenCL C program text be compiled as C++ so that the
// reference's own kernels (kernels/uppe.cl, fft.cl, ionization.cl, paraxial.cl) run on host cores.
// Nothing in the product links or includes this file.
//
// Supplies what those kernels use from OpenCL C: the double2 vector type with .s0/.s1 and the
// arithmetic operators, the address-space qualifiers (empty here), and the work-item functions
// get_global_id / get_global_size, which read per-thread state set by the generated launchers.
#pragma once
#include <cmath>
#include <cstdint>

struct double2 {
    double s0, s1;
    double2() : s0(0.0), s1(0.0) {}
    double2(double a, double b) : s0(a), s1(b) {}
    double2& operator+=(const double2& o) { s0 += o.s0; s1 += o.s1; return *this; }
    double2& operator-=(const double2& o) { s0 -= o.s0; s1 -= o.s1; return *this; }
    double2& operator*=(double f) { s0 *= f; s1 *= f; return *this; }
    double2& operator/=(double f) { s0 /= f; s1 /= f; return *this; }
};
inline double2 operator+(const double2& a, const double2& b) { return double2(a.s0 + b.s0, a.s1 + b.s1); }
inline double2 operator-(const double2& a, const double2& b) { return double2(a.s0 - b.s0, a.s1 - b.s1); }
inline double2 operator-(const double2& a) { return double2(-a.s0, -a.s1); }
inline double2 operator*(const double2& a, double f) { return double2(a.s0 * f, a.s1 * f); }
inline double2 operator*(double f, const double2& a) { return double2(a.s0 * f, a.s1 * f); }
inline double2 operator/(const double2& a, double f) { return double2(a.s0 / f, a.s1 / f); }

#define __kernel
#define __global
#define __local
#define __constant static const

// Work-item state of the calling host thread (one work item at a time per thread).
static thread_local long clshim_gid[3];
static thread_local long clshim_gsize[3];
static inline int get_global_id(int d) { return (int)clshim_gid[d]; }
static inline int get_global_size(int d) { return (int)clshim_gsize[d]; }
