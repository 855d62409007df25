// pd_math.cuh -- small device helpers with the reference's FP64 evaluation order.
// Everything here is compiled with -fmad=false so that a*b+c stays a rounded multiply
// followed by a rounded add, as in the reference's compiled CPU code.
#ifndef PD_MATH_CUH
#define PD_MATH_CUH
#include <stdint.h>

namespace pdg {

struct D3 {
  double x, y, z;
};

__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double comp(const D3 &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ void set_comp(D3 &a, int k, double v) {
  if (k == 0) a.x = v;
  else if (k == 1) a.y = v;
  else a.z = v;
}
// Eigen 3.3 reduction order for a 1x3 row: (x0 + x1) + x2.
__device__ __forceinline__ double sq3(D3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
__device__ __forceinline__ double norm3(D3 a) { return sqrt(sq3(a)); }
__device__ __forceinline__ double dot3(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// a / b, correctly rounded, from rb = RN(1/b): one correction step with an exact
// remainder (Markstein's theorem: if rb is within half an ulp of 1/b and q0 within one
// ulp of a/b, then RN(q0 + (a - b*q0)*rb) = RN(a/b)). Used where one divisor serves
// several dividends; tests compare the whole step with the FP64 oracle bit for bit.
__device__ __forceinline__ double div_rcp(double a, double b, double rb) {
  double q0 = a * rb;
  double r = fma(-q0, b, a);
  return fma(r, rb, q0);
}

// Order-preserving map of doubles onto unsigned 64-bit keys (for atomic min/max).
__device__ __forceinline__ unsigned long long ord_key(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double ord_val(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double d;
  memcpy(&d, &u, 8);
  return d;
}

}  // namespace pdg
#endif
