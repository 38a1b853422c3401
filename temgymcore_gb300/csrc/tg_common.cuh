// tg_common.cuh - shared definitions of the sm_103a ray-chain kernels.
//
// A model (list of tg_component, host float64) is compiled on the host into
// a Program: a flat list of steps.  Every component contributes two steps,
// in the order of run.py:75-82: a free-space propagator over
// (component.z - ray.z), then the component itself.  Because all rays share
// the same z after the first propagator, every propagation distance after the
// first is uniform; the compiler resolves them in float64 on the host and the
// device applies them in float32.  The uniform part of the pathlength
// (sum of distances) is accumulated on the host in float64; the per-ray part
// (lens / deflector / biprism terms) is accumulated on the device in float32
// and added to the float64 pathlength once per ray.
//
// The Program travels as a __grid_constant__ kernel parameter (constant
// bank), so every thread reads the same step descriptor with a broadcast.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/temgym_gb300.h"
#include "aberration.cuh"

namespace tg {

enum OpKind : int32_t {
  OP_NOP = 0,
  OP_FREE = 1,       // c0 = d
  OP_FREE_VARZ = 2,  // first propagator with per-ray z: d_i = zc - z_i
  OP_LENS = 3,       // c0 = 1/f, c1 = 1/(2f)
  OP_SHIFT = 4,      // c0..c3 = dx, dy, ddx, ddy (scanner / descanner)
  OP_DEFLECT = 5,    // c0, c1 = def_x, def_y; pl += dx*x + dy*y (incoming)
  OP_BIPRISM = 6,    // c0 = def_x;   dx += def_x*sign(x); pl += dx*x + dy*y
  OP_ROTATE = 7,     // c0 = cos, c1 = sin
  OP_APERTURE = 8,   // c0 = r^2, c1 = cx, c2 = cy
  OP_PROBE_SHIFT = 9, // per-probe shift: Delta = K (4x2) sp + k0 (float64 in pcoef)
  OP_ABER = 10       // aberrated lens: c0 = 1/f, c1 = 1/(2f); aux = Program::aber slot
};

struct Op {
  int32_t kind;
  int32_t aux;   // OP_PROBE_SHIFT: index into Program::pcoef; OP_BIPRISM: sign-bit slot
  float c[6];
};

constexpr int kMaxSteps = 2 * TG_MAX_COMPONENTS;
constexpr int kMaxProbeOps = 8;

struct Program {
  int32_t n_steps;
  int32_t n_biprism;
  int32_t has_aperture;
  int32_t n_probe_ops;
  int32_t n_aber;     // aberrated lenses (OP_ABER); not supported by the adjoint paths
  int32_t dircos;     // free-space steps use direction cosines (Op::aux = 1 on them)
  double zc_first;    // z of the first component (OP_FREE_VARZ)
  double pl_const;    // float64 sum of the uniform distances
  double z_out;       // uniform output z
  double pcoef[kMaxProbeOps][12];  // per-probe shift: rows (x,y,dx,dy) x (spx, spy, 1)
  Op op[kMaxSteps];
  double dstep[kMaxSteps];  // float64 distance of each propagator step (0 elsewhere)
  int32_t comp_kind[kMaxSteps];  // tg_kind of the component behind each step (-1 = propagator)
  float aber[kMaxAber][kAberFloats];  // per aberrated lens: W, dW/dx, dW/dy monomials
};

// Host-side compilation (model.cpp).  per_ray_z: input z is a per-ray array.
int compile_program(const tg_model* model, bool per_ray_z, double z_scalar,
                    Program* prog);

// Float64 5x5 affine matrix of one linear component over (x, y, dx, dy, 1)
// (host).  A biprism gives the identity: its offset def_x * sign(x) depends
// on the ray.  TG_ERR_UNSUPPORTED for a nonlinear or per-probe component.
int component_affine_f64(const tg_component& c, double cm[25]);

// Device error word: one per translation unit; tg_get_error_word ORs them.
#define TG_DEFINE_ERROR_WORD(tu)                                             \
  static __device__ uint32_t g_tg_err;                                       \
  extern "C" int tg_internal_err_##tu(uint32_t* out, int clear) {            \
    uint32_t v = 0;                                                          \
    if (cudaMemcpyFromSymbol(&v, g_tg_err, sizeof(v)) != cudaSuccess)        \
      return TG_ERR_CUDA;                                                    \
    *out |= v;                                                               \
    if (clear) {                                                             \
      uint32_t z = 0;                                                        \
      if (cudaMemcpyToSymbol(g_tg_err, &z, sizeof(z)) != cudaSuccess)        \
        return TG_ERR_CUDA;                                                  \
    }                                                                        \
    return TG_OK;                                                            \
  }

__device__ __forceinline__ float sgnf(float v) {
  return v > 0.f ? 1.f : (v < 0.f ? -1.f : 0.f);
}

// ---------------------------------------------------------------- binning
// metres -> pixel index, bit-exact with the float64 reference arithmetic
// ((m0*a + m1*b) + m2, no FMA, rint half-to-even, saturating int32, NaN->0).
// Fast path: float32 evaluation with a rigorous error bound; a value whose
// distance to the nearest half-integer is within the bound (or that is
// large / non-finite) is recomputed exactly in float64.  Ties are therefore
// decided by the float64 path, so the result equals the float64 result.
struct BinCoef {
  float f[6];
  double d[6];
};

__device__ __forceinline__ int bin_exact64(float af, float bf, double m0,
                                           double m1, double m2) {
  // the conversions sit in volatile blocks, so that the compiler keeps them
  // behind the caller's branch instead of running them for every thread
  double a, b;
  asm volatile("cvt.f64.f32 %0, %1;" : "=d"(a) : "f"(af));
  asm volatile("cvt.f64.f32 %0, %1;" : "=d"(b) : "f"(bf));
  double v = __dadd_rn(__dadd_rn(__dmul_rn(m0, a), __dmul_rn(m1, b)), m2);
  if (v != v) return 0;       // NaN -> 0 (the hardware conversion gives INT_MIN)
  return __double2int_rn(v);  // cvt.rni.s32.f64: saturating
}

__device__ __forceinline__ int bin_one(float a, float b, float m0, float m1,
                                       float m2, double d0, double d1,
                                       double d2) {
  float p0 = m0 * a, p1 = m1 * b;
  float v = (p0 + p1) + m2;
  float s = fabsf(p0) + fabsf(p1) + fabsf(m2);
  // |v - exact| <= ~5 * 2^-24 * s; use 2^-19 * s (16x margin) + denormal guard
  float bound = s * 1.9073486e-06f + 1e-30f;
  // nearest integer by the 1.5 * 2^23 constant (float32 ulp 1 there, exact
  // for |v| < 2^22), so no conversion instruction runs; r = v - rint(v)
  // exactly, and 1/2 - |r| is the distance to the nearest half-integer
  const float magic = 12582912.f;
  const float t = __fadd_rn(v, magic);
  const float r = __fsub_rn(v, __fsub_rn(t, magic));
  bool ok = (fabsf(v) < 4194304.f) && (0.5f - fabsf(r) > bound);  // |v| < 2^22, finite
  if (ok) return __float_as_int(t) - __float_as_int(magic);
  return bin_exact64(a, b, d0, d1, d2);
}

__device__ __forceinline__ void bin_yx(float x, float y, const BinCoef& bc,
                                       int& py, int& px) {
  py = bin_one(y, x, bc.f[0], bc.f[1], bc.f[2], bc.d[0], bc.d[1], bc.d[2]);
  px = bin_one(y, x, bc.f[3], bc.f[4], bc.f[5], bc.d[3], bc.d[4], bc.d[5]);
}

inline BinCoef make_bincoef(const tg_grid* g) {
  BinCoef b;
  for (int i = 0; i < 6; ++i) {
    b.d[i] = g->m[i];
    b.f[i] = (float)g->m[i];
  }
  return b;
}

// Warp-aggregated histogram increment: lanes hitting the same bin combine
// into one atomic issued by the lowest lane (all 32 lanes must call).
template <typename CountT>
__device__ __forceinline__ void hist_add_warp(CountT* hist, int bin, bool valid) {
  unsigned key = valid ? (unsigned)bin : 0xffffffffu;
  unsigned peers = __match_any_sync(0xffffffffu, key);
  int lane = threadIdx.x & 31;
  if (valid && lane == (__ffs(peers) - 1)) {
    unsigned cnt = __popc(peers);
    if constexpr (sizeof(CountT) == 8)
      atomicAdd(reinterpret_cast<unsigned long long*>(hist) + bin,
                (unsigned long long)cnt);
    else
      atomicAdd(reinterpret_cast<unsigned int*>(hist) + bin, cnt);
  }
}

// Exact float -> double conversion with integer operations (the hardware
// conversion issues on the float64 pipe, ~1/64 of the float32 rate on GB300):
// normal numbers rebias the exponent and widen the mantissa; zeros, denormals,
// infinities and NaNs take the hardware conversion.
__device__ __forceinline__ double f32_to_f64(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)v;
  const uint64_t d = ((uint64_t)(b >> 31) << 63) | ((uint64_t)(e + (1023u - 127u)) << 52) |
                     ((uint64_t)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}

// m / 2^a rounded half-even (m < 2^24, 1 <= a <= 26); tie: exactly halfway.
__device__ __forceinline__ long long rne_shr(uint32_t m, int a, bool& tie) {
  const uint32_t q = m >> a, rem = m & ((1u << a) - 1u), half = 1u << (a - 1);
  tie = rem == half;
  return (long long)(q + ((rem > half || (tie && (q & 1u))) ? 1u : 0u));
}

// b + p rounded to nearest even, bit-identical to __dadd_rn(b, (double)p),
// with integer operations in the usual case (a metre-scale float64 base plus
// a float32 per-ray part): GB300 runs float64 at ~1/64 of the float32 rate.
// With u = ulp(b) = 2^(e_b - 1075) and p = m 2^(e_p - 150) (m its 24-bit
// significand), p / u = m 2^sh, sh = e_p - e_b + 925: a shift of m, exact
// for sh >= 0 and rounded half-even for sh < 0.  Adding n = round(p / u) to
// b's bit pattern adds it to b's 53-bit integer significand, which is the
// correctly rounded sum while the result keeps b's exponent (or lands on the
// next power of two).  When it would land on or below b's binade's lower
// boundary the grid below is twice as fine: the sum is rounded at u / 2
// instead (n2 = round(2 p / u)), and the bits follow from b's mantissa field
// f as bits(b) + f + n2 (or the power of two itself when that rounding
// stays on it).  The float64 add is kept for zero, denormal and non-finite
// operands, b outside 2^-1021..2^1022, |p| beyond ~|b|, exact halfway
// cases (ties go to the even significand of the sum, not of n) and sums
// that leave the binade further.
__device__ __forceinline__ double add_f64_f32(double b, float p) {
  const long long bb = __double_as_longlong(b);
  const uint32_t pb = __float_as_uint(p);
  const int eb = (int)((bb >> 52) & 0x7ff), ep = (int)((pb >> 23) & 0xffu);
  if (eb >= 2 && eb <= 2045) {
    if ((pb & 0x7fffffffu) == 0u) return b;  // b + (+-0)
    const int sh = ep - eb + 925;
    if (ep >= 1 && ep <= 254 && sh <= 29) {
      const uint32_t m = (pb & 0x7fffffu) | 0x800000u;
      long long n = 0, n2 = 0;  // p / u and 2 p / u, rounded half-even
      bool tie = false, tie2 = false;
      if (sh >= 0) {
        n = (long long)m << sh;
        n2 = n << 1;
      } else if (sh >= -26) {  // below: |p / u| < 1/8, both round to 0
        n = rne_shr(m, -sh, tie);
        n2 = sh == -1 ? (long long)m : rne_shr(m, -sh - 1, tie2);
      }
      const bool neg = ((pb >> 31) != 0u) != (bb < 0);  // the magnitude of b shrinks
      const long long N = neg ? -n : n, N2 = neg ? -n2 : n2;
      const long long f = bb & 0xfffffffffffffLL;
      if (f + N >= 1) {  // inside the binade, or onto the next power of two
        if (!tie && f + N <= (1LL << 52)) return __longlong_as_double(bb + N);
      } else {  // at or below the binade's lower boundary: the finer grid
        const long long low = 2 * f + N2;
        if (!tie && !tie2 && low >= -(1LL << 52))
          return __longlong_as_double(low >= 0 ? bb - f : bb + f + N2);
      }
    }
  }
  // the float64 add in a volatile block, so that the compiler does not run
  // it (conversion + add) ahead of the branch for every thread
  double r;
  asm volatile("{\n\t.reg .f64 pd;\n\tcvt.f64.f32 pd, %2;\n\tadd.rn.f64 %0, %1, pd;\n\t}"
               : "=d"(r) : "d"(b), "f"(p));
  return r;
}

// ---------------------------------------------------------------- mbarriers
// Shared-memory mbarriers for TMA copies and tensor-core commits.  Every wait
// is bounded: after kWaitCycles the caller gets false and the error word its
// translation unit passes in receives the given bit.
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}

// Per-thread asynchronous 16-byte copy global -> shared (cached in L2 only);
// both addresses 16-byte aligned.  A thread that reads back only the slots it
// filled itself needs no barrier: cp_async_wait orders its own copies.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, uint32_t* err,
                                          uint32_t bit) {
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try(a, parity)) return true;
    if ((it & 255u) == 255u && clock64() - t0 > kWaitCycles) {
      atomicOr(err, bit);
      return false;
    }
  }
}

// ---------------------------------------------------------------- ray ops
struct RayS {
  float x, y, dx, dy, plv;  // plv: per-ray (varying) pathlength part
};

// Aberrated lens (components.py:193-215): thin lens to the ideal slopes u,
// then the slope kick -grad W(u) / f and the pathlength + W(u) / f, with W the
// Krivanek polynomial of one Program::aber slot.
__device__ __forceinline__ void aber_forward(const float* a, float k1, float h, RayS& r) {
  const float x = r.x, y = r.y;
  const float ux = fmaf(-x, k1, r.dx), uy = fmaf(-y, k1, r.dy);
  const float W = tri_eval<6>(a, ux, uy);
  const float Wx = tri_eval<5>(a + kAberW, ux, uy);
  const float Wy = tri_eval<5>(a + kAberW + kAberG, ux, uy);
  r.plv = fmaf(W, k1, r.plv - (x * x + y * y) * h);
  r.dx = fmaf(-Wx, k1, ux);
  r.dy = fmaf(-Wy, k1, uy);
}

// Apply one forward step.  dvar is the ray's own first distance (OP_FREE_VARZ
// only: component z minus the ray's z, formed in float64 by the caller once
// per ray, outside the step loop); pshift holds the current probe's shifts
// (OP_PROBE_SHIFT only); aber the Program's aberration polynomials (OP_ABER
// only, may be NULL otherwise).  sbits records biprism signs (2 bits per
// biprism: 1 = +, 2 = -) and alive is cleared by apertures.  No float64
// arithmetic runs per step.
__device__ __forceinline__ void op_forward(const Op& op, const float4* pshift,
                                           RayS& r, float dvar, uint64_t& sbits,
                                           bool& alive, const float* aber = nullptr) {
  switch (op.kind) {
    case OP_FREE:
    case OP_FREE_VARZ: {
      const float d = op.kind == OP_FREE ? op.c[0] : dvar;
      if (op.aux) {  // direction cosines (propagator.py:100-110): x += d dx / N^2, pl += d N
        const float s2 = fmaf(r.dx, r.dx, r.dy * r.dy);
        const float n2 = 1.f + s2;
        const float t = d / n2;
        r.x = fmaf(r.dx, t, r.x);
        r.y = fmaf(r.dy, t, r.y);
        r.plv = fmaf(d, s2 / (sqrtf(n2) + 1.f), r.plv);  // d (N - 1); the uniform d is float64
      } else {
        r.x = fmaf(r.dx, d, r.x);
        r.y = fmaf(r.dy, d, r.y);
      }
    } break;
    case OP_LENS: {
      float x = r.x, y = r.y;
      r.plv = fmaf(-fmaf(x, x, y * y), op.c[1], r.plv);
      r.dx = fmaf(-x, op.c[0], r.dx);
      r.dy = fmaf(-y, op.c[0], r.dy);
    } break;
    case OP_SHIFT:
      r.x += op.c[0];
      r.y += op.c[1];
      r.dx += op.c[2];
      r.dy += op.c[3];
      break;
    case OP_PROBE_SHIFT: {  // per-probe constants staged in shared memory
      float4 s = pshift[op.aux];
      r.x += s.x;
      r.y += s.y;
      r.dx += s.z;
      r.dy += s.w;
    } break;
    case OP_DEFLECT: {
      r.plv += fmaf(r.dx, r.x, r.dy * r.y);
      r.dx += op.c[0];
      r.dy += op.c[1];
    } break;
    case OP_BIPRISM: {
      r.plv += fmaf(r.dx, r.x, r.dy * r.y);
      float s = sgnf(r.x);
      sbits |= (uint64_t)(s > 0.f ? 1u : (s < 0.f ? 2u : 0u)) << (2 * op.aux);
      r.dx = fmaf(op.c[0], s, r.dx);
    } break;
    case OP_ROTATE: {
      float c = op.c[0], s = op.c[1];
      float x = r.x, y = r.y, dx = r.dx, dy = r.dy;
      r.x = fmaf(x, c, -(y * s));
      r.y = fmaf(x, s, y * c);
      r.dx = fmaf(dx, c, -(dy * s));
      r.dy = fmaf(dx, s, dy * c);
    } break;
    case OP_APERTURE: {
      float ex = r.x - op.c[1], ey = r.y - op.c[2];
      if (!(fmaf(ex, ex, ey * ey) < op.c[0])) alive = false;
    } break;
    case OP_ABER:
      if (aber) aber_forward(aber + op.aux * kAberFloats, op.c[0], op.c[1], r);
      break;
    default:
      break;
  }
}

// ---------------------------------------------------------------- adjoint
struct Adj {
  float lx, ly, ldx, ldy, lpl;
};

// Reverse of the aberrated lens (aber_forward): q is the state entering the
// lens (the caller recomputes it: the slope map u -> u - grad W(u) / f has no
// closed-form inverse), a the adjoint after the lens, turned into the adjoint
// before it; c0 receives d L / d f.  With u = d - r / f:
//   d(d')/du = I - H / f (H the Hessian of W at u), d pl' / du = grad W / f,
//   d(d')/d(1/f) = -r - grad W + (H r) / f, d pl'/d(1/f) = W - (grad W . r) / f,
//   d pl' / d(1/(2f)) = -(x^2 + y^2).
__device__ __forceinline__ void aber_reverse(const float* aw, float k1, float h, const RayS& q, Adj& ad,
                                             float& c0) {
  const float x = q.x, y = q.y;
  const float ux = fmaf(-x, k1, q.dx), uy = fmaf(-y, k1, q.dy);
  const float W = tri_eval<6>(aw, ux, uy);
  float Wx, Hxx, Hxy1, Wy, Hxy2, Hyy;
  tri_eval_d<5>(aw + kAberW, ux, uy, &Wx, &Hxx, &Hxy1);
  tri_eval_d<5>(aw + kAberW + kAberG, ux, uy, &Wy, &Hxy2, &Hyy);
  const float Hxy = 0.5f * (Hxy1 + Hxy2);
  const float ldx = ad.ldx, ldy = ad.ldy, lpl = ad.lpl;
  const float lux = ldx * (1.f - k1 * Hxx) - ldy * (k1 * Hxy) + lpl * k1 * Wx;
  const float luy = -ldx * (k1 * Hxy) + ldy * (1.f - k1 * Hyy) + lpl * k1 * Wy;
  const float dk1 = ldx * (-x - Wx + k1 * (Hxx * x + Hxy * y)) + ldy * (-y - Wy + k1 * (Hxy * x + Hyy * y)) +
                    lpl * (W - k1 * (Wx * x + Wy * y));
  const float dh = -lpl * (x * x + y * y);
  c0 = -k1 * k1 * (dk1 + 0.5f * dh);
  ad.ldx = lux;
  ad.ldy = luy;
  ad.lx = ad.lx - k1 * lux - 2.f * h * x * lpl;
  ad.ly = ad.ly - k1 * luy - 2.f * h * y * lpl;
}

// Reverse one step: on entry r is the state after the step and a the adjoint
// after it; on exit both describe the state before it.  c receives the step's
// parameter sensitivities for this ray.  gz receives dL/dz_in (OP_FREE_VARZ).
__device__ __forceinline__ void op_reverse(const Op& op, const float4* pshift, RayS& r,
                                           Adj& a, uint64_t sbits, float dvar,
                                           float c[4], float& gz) {
  switch (op.kind) {
    case OP_FREE:
    case OP_FREE_VARZ: {
      float d = (op.kind == OP_FREE) ? op.c[0] : dvar;
      if (op.aux) {  // direction cosines: slopes unchanged, so the step inverts exactly
        const float dx = r.dx, dy = r.dy;
        const float n2 = 1.f + fmaf(dx, dx, dy * dy);  // as in the forward step
        const float inv = 1.f / n2, nn = sqrtf(n2);
        const float g = (a.lx * dx + a.ly * dy) * inv + a.lpl * nn;
        c[0] = g;
        if (op.kind == OP_FREE_VARZ) gz = -g;
        const float t = d / n2;
        r.x = fmaf(-dx, t, r.x);
        r.y = fmaf(-dy, t, r.y);
        // d x'/d dx = d (1/n2 - 2 dx^2/n2^2), d x'/d dy = -2 d dx dy / n2^2, d pl'/d dx = d dx / N
        const float di = d * inv, di2 = 2.f * di * inv;
        const float jxx = di - di2 * dx * dx, jyy = di - di2 * dy * dy, jxy = -di2 * dx * dy;
        const float pn = d / nn;
        a.ldx += a.lx * jxx + a.ly * jxy + a.lpl * pn * dx;
        a.ldy += a.lx * jxy + a.ly * jyy + a.lpl * pn * dy;
      } else {
        float g = a.lx * r.dx + a.ly * r.dy + a.lpl;
        c[0] = g;
        if (op.kind == OP_FREE_VARZ) gz = -g;
        r.x = fmaf(-r.dx, d, r.x);
        r.y = fmaf(-r.dy, d, r.y);
        a.ldx = fmaf(a.lx, d, a.ldx);
        a.ldy = fmaf(a.ly, d, a.ldy);
      }
    } break;
    case OP_LENS: {
      float k = op.c[0], h = op.c[1];
      float x = r.x, y = r.y;
      r.dx = fmaf(x, k, r.dx);
      r.dy = fmaf(y, k, r.dy);
      c[0] = (a.ldx * x + a.ldy * y) * (k * k) + a.lpl * (x * x + y * y) * (k * h);
      a.lx = a.lx - a.ldx * k - a.lpl * 2.f * x * h;
      a.ly = a.ly - a.ldy * k - a.lpl * 2.f * y * h;
    } break;
    case OP_SHIFT:
    case OP_PROBE_SHIFT: {
      float4 s = (op.kind == OP_SHIFT) ? make_float4(op.c[0], op.c[1], op.c[2], op.c[3])
                                       : pshift[op.aux];
      r.x -= s.x; r.y -= s.y; r.dx -= s.z; r.dy -= s.w;
      c[0] = a.lx; c[1] = a.ly; c[2] = a.ldx; c[3] = a.ldy;
    } break;
    case OP_DEFLECT: {
      c[0] = a.ldx;
      c[1] = a.ldy;
      r.dx -= op.c[0];
      r.dy -= op.c[1];
      a.lx = fmaf(a.lpl, r.dx, a.lx);
      a.ly = fmaf(a.lpl, r.dy, a.ly);
      a.ldx = fmaf(a.lpl, r.x, a.ldx);
      a.ldy = fmaf(a.lpl, r.y, a.ldy);
    } break;
    case OP_BIPRISM: {
      uint32_t b = (uint32_t)(sbits >> (2 * op.aux)) & 3u;
      float s = b == 1u ? 1.f : (b == 2u ? -1.f : 0.f);
      c[0] = a.ldx * s;
      r.dx = fmaf(-op.c[0], s, r.dx);
      a.lx = fmaf(a.lpl, r.dx, a.lx);
      a.ly = fmaf(a.lpl, r.dy, a.ly);
      a.ldx = fmaf(a.lpl, r.x, a.ldx);
      a.ldy = fmaf(a.lpl, r.y, a.ldy);
    } break;
    case OP_ROTATE: {
      float cs = op.c[0], sn = op.c[1];
      c[0] = -a.lx * r.y + a.ly * r.x - a.ldx * r.dy + a.ldy * r.dx;
      float x = r.x, y = r.y, dx = r.dx, dy = r.dy;
      r.x = x * cs + y * sn;
      r.y = -x * sn + y * cs;
      r.dx = dx * cs + dy * sn;
      r.dy = -dx * sn + dy * cs;
      float lx = a.lx, ly = a.ly, ldx = a.ldx, ldy = a.ldy;
      a.lx = lx * cs + ly * sn;
      a.ly = -lx * sn + ly * cs;
      a.ldx = ldx * cs + ldy * sn;
      a.ldy = -ldx * sn + ldy * cs;
    } break;
    default:
      break;
  }
}

}  // namespace tg
