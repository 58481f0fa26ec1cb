/*
 * Forward-mode dual numbers for the tangent-linear build of the oracle (TEST
 * INFRASTRUCTURE ONLY): oracle/Makefile compiles ns.c, ib.c and embedded.c a second
 * time as C++ with this header forced in front, so that every `double` of those
 * restated kernels becomes a dual_t (value v, derivative d).  Each arithmetic
 * operation then also carries the derivative of its result along one direction of the
 * inputs (the chain rule applied operation by operation), which turns the restated
 * step into its exact tangent-linear model: the FP64 tangent-linear reference the GPU
 * adjoint is checked against.  Comparisons look at values only, so the branches (the
 * tagging decisions, the reference's own control flow) are those of the plain build.
 *
 * A dual_t array has the memory layout of numpy's complex128 (real = value,
 * imaginary = derivative), which is how oracle/__init__.py passes them.
 */
#ifndef ORACLE_DUAL_H
#define ORACLE_DUAL_H
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

struct dual_t {
    double v, d;
    dual_t() : v(0), d(0) {}
    dual_t(double a) : v(a), d(0) {}
    dual_t(double a, double b) : v(a), d(b) {}
    explicit operator int() const { return (int)v; }
    dual_t &operator+=(const dual_t &o) { v += o.v; d += o.d; return *this; }
    dual_t &operator-=(const dual_t &o) { v -= o.v; d -= o.d; return *this; }
    dual_t &operator*=(const dual_t &o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
    dual_t &operator/=(const dual_t &o) { *this = dual_t(v / o.v, (d * o.v - v * o.d) / (o.v * o.v)); return *this; }
};

static inline dual_t operator+(dual_t a, dual_t b) { return dual_t(a.v + b.v, a.d + b.d); }
static inline dual_t operator-(dual_t a, dual_t b) { return dual_t(a.v - b.v, a.d - b.d); }
static inline dual_t operator-(dual_t a) { return dual_t(-a.v, -a.d); }
static inline dual_t operator*(dual_t a, dual_t b) { return dual_t(a.v * b.v, a.d * b.v + a.v * b.d); }
static inline dual_t operator/(dual_t a, dual_t b)
{
    return dual_t(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v));
}
static inline bool operator<(dual_t a, dual_t b) { return a.v < b.v; }
static inline bool operator>(dual_t a, dual_t b) { return a.v > b.v; }
static inline bool operator<=(dual_t a, dual_t b) { return a.v <= b.v; }
static inline bool operator>=(dual_t a, dual_t b) { return a.v >= b.v; }
static inline bool operator==(dual_t a, dual_t b) { return a.v == b.v; }
static inline bool operator!=(dual_t a, dual_t b) { return a.v != b.v; }
static inline bool operator!(dual_t a) { return !a.v; }

static inline dual_t sqrt(dual_t a)
{
    const double s = sqrt(a.v);
    return dual_t(s, a.d / (2 * s));
}
static inline dual_t fabs(dual_t a) { return a.v < 0 ? -a : a; }
static inline dual_t pow(dual_t a, int n)
{
    return n == 2 ? a * a : dual_t(pow(a.v, n), n * pow(a.v, n - 1) * a.d);
}
static inline dual_t pow(dual_t a, double e) { return dual_t(pow(a.v, e), e * pow(a.v, e - 1) * a.d); }
static inline dual_t sin(dual_t a) { return dual_t(sin(a.v), cos(a.v) * a.d); }
static inline dual_t cos(dual_t a) { return dual_t(cos(a.v), -sin(a.v) * a.d); }
static inline dual_t tan(dual_t a)
{
    const double t = tan(a.v);
    return dual_t(t, (1 + t * t) * a.d);
}
static inline dual_t acos(dual_t a) { return dual_t(acos(a.v), -a.d / sqrt(1 - a.v * a.v)); }
static inline dual_t asin(dual_t a) { return dual_t(asin(a.v), a.d / sqrt(1 - a.v * a.v)); }

#define double dual_t
#endif
