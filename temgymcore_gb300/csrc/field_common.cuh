// field_common.cuh - per-beam coefficient records of the Gaussian-beamlet
// detector field (gaussian.py:225-369) shared by the prep kernel, the direct
// kernels and the separable tensor-core path.
//
// For each beam the prep kernel reduces the reference's per-pixel formula
//   field(r2) = pref * exp(i (k/2) (s^T Q2 s + phi1(s) - phi2(s) + 2 s.f) + i k pl),
//   s = r2 - e,  (gaussian.py:276-316)
// to a complex quadratic polynomial in the integer pixel indices:
//   Phi(row, col) = c_cc col^2 + c_rr row^2 + c_rc row col + c_c col + c_r row + c_0.
// Because col^2, row^2, row*col, col, row are integers, reducing each real
// coefficient modulo one turn commutes with the evaluation.  The real parts
// (the phase) are therefore stored as 64-bit fixed-point fractions of a turn
// (2^64 = one turn) and evaluated with wrap-around integer arithmetic, exact
// to 2^-64 turn; the float64 pathlength phase k*pl enters the constant after
// an exact (FMA TwoProduct + two-part 2*pi) reduction.  The imaginary parts
// (the Gaussian envelope) become a float32 log-amplitude quadratic centred on
// the envelope maximum.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "tg_common.cuh"

namespace tg {

// exp(logamp) * exp(i 2 pi turns / 2^64), the angle from the top 32 bits of
// the turn fraction (signed): [-pi, pi).
__device__ __forceinline__ float2 cexpf_turn(float logamp, uint64_t turns) {
  int32_t hi = (int32_t)(turns >> 32);
  float ang = (float)hi * 1.4629180792671596e-09f;  // 2*pi / 2^32
  float s, c;
  __sincosf(ang, &s, &c);
  float a = __expf(logamp);
  return make_float2(a * c, a * s);
}

// One separable operand value (a beam's row or column factor) at the integer
// line g: exp(e0 - (bq d^2 + bl d) + i 2 pi th / 2^64) with d = g - cen and
// th the exact fixed-point phase at g.
__device__ __forceinline__ float2 sep_operand(float e0, float bq, float bl, float cen, int g,
                                              uint64_t th) {
  const float d = (float)g - cen;
  return cexpf_turn(fmaf(-d, fmaf(bq, d, bl), e0), th);
}

// bf16 hi and lo parts of two floats (hi = bf16(v), lo = bf16(v - hi), both
// round-to-nearest-even), each pair packed with a in the low half.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - __low2float(h), b - __high2float(h));
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Fast record (fixed-point phase, float32 envelope), 96 bytes.
struct alignas(16) BeamFast {
  uint64_t p_cc, p_rr, p_rc, p_c, p_r, p_0;  // turns * 2^64
  float r0, c0;          // envelope centre (row, col)
  float e0;              // log-amplitude at the centre
  float b_cc, b_rr, b_rc, l_c, l_r;  // log-amp = e0 - (b_cc dc^2 + b_rr dr^2 + b_rc dr dc + l_c dc + l_r dr)
  float rho_re, rho_im;  // exp(-2 b_cc + i 2pi (2 p_cc)): column-step ratio of ratios
};

// float64 record for the all-float64 comparator kernel, 128 bytes.
struct alignas(16) BeamF64 {
  double re[6];   // c_cc, c_rr, c_rc, c_c, c_r, c_0 real parts (radians)
  double im[6];   // imaginary parts
  double ph0;     // exactly reduced k*pl + arg(pref), radians
  double lnamp;   // ln |pref|
  double pad[2];
};

// Float64 model of the per-beam preparation: two steps per component (the
// free-space distance, then the component), as run.py:75-82 inserts them.
enum DKind : int32_t { D_NOP = 0, D_FREE = 1, D_LENS = 2, D_SHIFT = 3, D_BIPRISM = 4, D_ROTATE = 5,
                       D_ABER = 6 };

struct DStep {
  int32_t kind;
  int32_t pad;
  double a[4];  // FREE: d; LENS: f, 1/f; SHIFT: x, y, dx, dy; BIPRISM: def_x; ROTATE: cos, sin; ABER: f
};

struct DModel {
  int32_t n;
  int32_t n_aber;
  DStep s[kMaxSteps];
  double aber[kMaxAber][kAberW];  // D_ABER (pad = slot): W monomials, float64
};

// Host: a tg_model (paraxial) -> DModel with the beams starting at z_in.
int build_dmodel(const tg_model* model, double z_in, DModel* dm);

// Host (field.cu): bytes of the per-beam records of n beams (BeamFast array at
// offset 0), and the records of the beams with every amplitude taken as 1.
size_t field_records_bytes(int64_t n);
int field_prep_unit_amp(const DModel& dm, const tg_beams* beams, const tg_pixel_map* pm, void* records,
                        size_t bytes, void* stream, int input_plane);

// Pixel map of the detector: pixels -> metres (grid.py:155-182).
struct PixMap {
  int32_t h, w;
  double t[6];  // y = (t0*row + t1*col) + t2 ; x = (t3*row + t4*col) + t5
};

}  // namespace tg
