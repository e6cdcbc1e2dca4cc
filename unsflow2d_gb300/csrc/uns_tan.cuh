// uns_tan.cuh -- forward-mode tangent numbers for the discrete adjoint.
//
// Tan carries a value and one directional derivative.  The physics functions
// of uns_phys.cuh are templates on their arithmetic type, so instantiating
// them on Tan and seeding one input direction at a time gives one column of
// their exact local Jacobian (no finite-difference step).  Branches
// (comparisons, fabs, the min/max of the limiter and the fluxes) follow the
// value, so the Jacobian is the one of the branch the forward pass took.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace uns {
// A namespace of its own, so that sqrt/fabs/pow of Tan are found only by
// argument-dependent lookup and never hide ::sqrt for doubles in namespace uns.
namespace ad {

struct Tan {
    double v, d;
    __host__ __device__ Tan() : v(0.0), d(0.0) {}
    __host__ __device__ Tan(double x) : v(x), d(0.0) {}
    __host__ __device__ Tan(double x, double dx) : v(x), d(dx) {}
};

__host__ __device__ __forceinline__ Tan operator+(Tan a, Tan b) { return Tan(a.v + b.v, a.d + b.d); }
__host__ __device__ __forceinline__ Tan operator-(Tan a, Tan b) { return Tan(a.v - b.v, a.d - b.d); }
__host__ __device__ __forceinline__ Tan operator-(Tan a) { return Tan(-a.v, -a.d); }
__host__ __device__ __forceinline__ Tan operator*(Tan a, Tan b) { return Tan(a.v * b.v, a.d * b.v + a.v * b.d); }
__host__ __device__ __forceinline__ Tan operator/(Tan a, Tan b) {
    double q = a.v / b.v;
    return Tan(q, (a.d - q * b.d) / b.v);
}
__host__ __device__ __forceinline__ Tan operator+(Tan a, double b) { return Tan(a.v + b, a.d); }
__host__ __device__ __forceinline__ Tan operator+(double a, Tan b) { return Tan(a + b.v, b.d); }
__host__ __device__ __forceinline__ Tan operator-(Tan a, double b) { return Tan(a.v - b, a.d); }
__host__ __device__ __forceinline__ Tan operator-(double a, Tan b) { return Tan(a - b.v, -b.d); }
__host__ __device__ __forceinline__ Tan operator*(Tan a, double b) { return Tan(a.v * b, a.d * b); }
__host__ __device__ __forceinline__ Tan operator*(double a, Tan b) { return Tan(a * b.v, a * b.d); }
__host__ __device__ __forceinline__ Tan operator/(Tan a, double b) { return Tan(a.v / b, a.d / b); }
__host__ __device__ __forceinline__ Tan operator/(double a, Tan b) {
    double q = a / b.v;
    return Tan(q, -q * b.d / b.v);
}
__host__ __device__ __forceinline__ Tan& operator+=(Tan& a, Tan b) { a = a + b; return a; }
__host__ __device__ __forceinline__ Tan& operator-=(Tan& a, Tan b) { a = a - b; return a; }
__host__ __device__ __forceinline__ Tan& operator*=(Tan& a, Tan b) { a = a * b; return a; }

__host__ __device__ __forceinline__ bool operator<(Tan a, Tan b) { return a.v < b.v; }
__host__ __device__ __forceinline__ bool operator>(Tan a, Tan b) { return a.v > b.v; }
__host__ __device__ __forceinline__ bool operator<=(Tan a, Tan b) { return a.v <= b.v; }
__host__ __device__ __forceinline__ bool operator>=(Tan a, Tan b) { return a.v >= b.v; }

__host__ __device__ __forceinline__ Tan sqrt(Tan a) {
    double r = ::sqrt(a.v);
    return Tan(r, a.d / (2.0 * r));
}
__host__ __device__ __forceinline__ Tan fabs(Tan a) { return a.v < 0.0 ? Tan(-a.v, -a.d) : a; }
// a^b for a > 0: d(a^b) = a^b (b' ln a + b a'/a).
__host__ __device__ __forceinline__ Tan pow(Tan a, Tan b) {
    double p = ::pow(a.v, b.v);
    double dd = b.v * a.d / a.v;
    if (b.d != 0.0) dd = dd + b.d * ::log(a.v);
    return Tan(p, p * dd);
}
__host__ __device__ __forceinline__ Tan pow(Tan a, double b) {
    double p = ::pow(a.v, b);
    return Tan(p, p * b * a.d / a.v);
}

}  // namespace ad
using ad::Tan;

// Value of a double or a Tan, for the few places that need the plain number.
__host__ __device__ __forceinline__ double val(double x) { return x; }
__host__ __device__ __forceinline__ double val(Tan x) { return x.v; }
__host__ __device__ __forceinline__ double der(Tan x) { return x.d; }

}  // namespace uns
