// Scalar types shared by the host driver and the sm_103a kernels.
//
// Real arithmetic runs in double (the JD outer loop) or float (the
// preconditioner under ICNTL(5)=1); complex arithmetic in the two-word
// structs zc (complex128) and cc (complex64), layout-compatible with
// std::complex and Fortran COMPLEX*16 / COMPLEX*8.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#define JD_HD __host__ __device__ __forceinline__

namespace jdg {

struct alignas(16) zc {
  double x, y;
  zc() = default;
  JD_HD zc(double r) : x(r), y(0) {}
  JD_HD zc(double r, double i) : x(r), y(i) {}
};
struct alignas(8) cc {
  float x, y;
  cc() = default;
  JD_HD cc(float r) : x(r), y(0) {}
  JD_HD cc(float r, float i) : x(r), y(i) {}
};

JD_HD zc operator+(zc a, zc b) { return zc(a.x + b.x, a.y + b.y); }
JD_HD zc operator-(zc a, zc b) { return zc(a.x - b.x, a.y - b.y); }
JD_HD zc operator-(zc a) { return zc(-a.x, -a.y); }
JD_HD zc operator*(zc a, zc b) { return zc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
JD_HD zc operator*(double s, zc a) { return zc(s * a.x, s * a.y); }
JD_HD zc operator*(zc a, double s) { return zc(s * a.x, s * a.y); }
JD_HD zc& operator+=(zc& a, zc b) { a.x += b.x; a.y += b.y; return a; }
JD_HD zc& operator-=(zc& a, zc b) { a.x -= b.x; a.y -= b.y; return a; }
JD_HD bool operator==(zc a, zc b) { return a.x == b.x && a.y == b.y; }
JD_HD cc operator+(cc a, cc b) { return cc(a.x + b.x, a.y + b.y); }
JD_HD cc operator-(cc a, cc b) { return cc(a.x - b.x, a.y - b.y); }
JD_HD cc operator-(cc a) { return cc(-a.x, -a.y); }
JD_HD bool operator==(cc a, cc b) { return a.x == b.x && a.y == b.y; }
JD_HD cc operator*(cc a, cc b) { return cc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
JD_HD cc operator*(float s, cc a) { return cc(s * a.x, s * a.y); }
JD_HD cc& operator+=(cc& a, cc b) { a.x += b.x; a.y += b.y; return a; }
JD_HD cc& operator-=(cc& a, cc b) { a.x -= b.x; a.y -= b.y; return a; }

JD_HD double rl(double a) { return a; }
JD_HD double rl(zc a) { return a.x; }
JD_HD float rl(float a) { return a; }
JD_HD float rl(cc a) { return a.x; }
JD_HD double cj(double a) { return a; }
JD_HD zc cj(zc a) { return zc(a.x, -a.y); }
JD_HD float cj(float a) { return a; }
JD_HD cc cj(cc a) { return cc(a.x, -a.y); }
JD_HD double ab2(double a) { return a * a; }
JD_HD double ab2(zc a) { return a.x * a.x + a.y * a.y; }
// fused a*b + c
JD_HD double fma_(double a, double b, double c) { return fma(a, b, c); }
JD_HD float fma_(float a, float b, float c) { return fmaf(a, b, c); }
JD_HD zc fma_(zc a, zc b, zc c) { return zc(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))); }
JD_HD cc fma_(cc a, cc b, cc c) { return cc(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y))); }

// storage <-> arithmetic conversions for the preconditioner precisions
template <class S> struct Arith { using type = S; };
template <> struct Arith<__nv_bfloat16> { using type = float; };
struct alignas(4) bc { __nv_bfloat16 x, y; };  // complex bf16 storage
template <> struct Arith<bc> { using type = cc; };

JD_HD double to_d(double a) { return a; }
JD_HD double to_d(float a) { return a; }
JD_HD zc to_z(zc a) { return a; }
JD_HD zc to_z(cc a) { return zc(a.x, a.y); }
template <class A, class B> struct Cvt;
template <> struct Cvt<double, double> { static JD_HD double f(double a) { return a; } };
template <> struct Cvt<float, double> { static JD_HD float f(double a) { return (float)a; } };
template <> struct Cvt<double, float> { static JD_HD double f(float a) { return a; } };
template <> struct Cvt<float, float> { static JD_HD float f(float a) { return a; } };
template <> struct Cvt<zc, zc> { static JD_HD zc f(zc a) { return a; } };
template <> struct Cvt<cc, zc> { static JD_HD cc f(zc a) { return cc((float)a.x, (float)a.y); } };
template <> struct Cvt<zc, cc> { static JD_HD zc f(cc a) { return zc(a.x, a.y); } };
template <> struct Cvt<cc, cc> { static JD_HD cc f(cc a) { return a; } };
template <class To, class From> JD_HD To cvt(From a) { return Cvt<To, From>::f(a); }

__device__ __forceinline__ float ld_arith(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ cc ld_arith(const bc* p) { bc v = *p; return cc(__bfloat162float(v.x), __bfloat162float(v.y)); }
__device__ __forceinline__ float ld_arith(const float* p) { return *p; }
__device__ __forceinline__ double ld_arith(const double* p) { return *p; }
__device__ __forceinline__ cc ld_arith(const cc* p) { return *p; }
__device__ __forceinline__ zc ld_arith(const zc* p) { return *p; }
// The same loads for factor entries and column indices streamed once per
// sweep: read-only path, no L1 allocation (L1 stays for the gathered vector).
__device__ __forceinline__ float ld_arith_nc(const float* p) {
  float r;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ double ld_arith_nc(const double* p) {
  double r;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(p));
  return r;
}
__device__ __forceinline__ float ld_arith_nc(const __nv_bfloat16* p) {
  unsigned short r;
  asm("ld.global.nc.L1::no_allocate.b16 %0, [%1];" : "=h"(r) : "l"(p));
  return __bfloat162float(__ushort_as_bfloat16(r));
}
__device__ __forceinline__ cc ld_arith_nc(const cc* p) {
  float x, y;
  asm("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(x), "=f"(y) : "l"(p));
  return cc(x, y);
}
__device__ __forceinline__ zc ld_arith_nc(const zc* p) {
  double x, y;
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "l"(p));
  return zc(x, y);
}
__device__ __forceinline__ cc ld_arith_nc(const bc* p) {
  unsigned short x, y;
  asm("ld.global.nc.L1::no_allocate.v2.b16 {%0, %1}, [%2];" : "=h"(x), "=h"(y) : "l"(p));
  return cc(__bfloat162float(__ushort_as_bfloat16(x)), __bfloat162float(__ushort_as_bfloat16(y)));
}
// a stored entry converted to the arithmetic type A
template <class A, class S> __device__ __forceinline__ A lda(const S* p) { return cvt<A>(ld_arith(p)); }
template <class A, class S> __device__ __forceinline__ A ldan(const S* p) { return cvt<A>(ld_arith_nc(p)); }
__device__ __forceinline__ int ld_idx_nc(const int* p) {
  int r;
  asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(r) : "l"(p));
  return r;
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}
#define CK(x) ::jdg::cuda_check((x), #x)

}  // namespace jdg
