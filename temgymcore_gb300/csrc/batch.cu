// batch.cu - many independent models with uneven component and ray counts in
// ONE persistent launch over a packed model table (forward + adjoint).
//
// The reference runs each model separately (run.py:85-116 per model, jax.grad
// per model); here the host packs every model into one device buffer (the
// plan): per-model records, a tile list and the adjoint coefficients.  A
// persistent grid pulls tiles (a model and a contiguous run of its rays) from
// an atomic work counter, stages that model's record in shared memory,
// evaluates the rays and writes the outputs.  Per-tile partials are reduced
// per model in a fixed order, so the results do not depend on which CTA took
// which tile.
//
// Closed-form forward.  Every supported step is affine in the ray state
// except the biprism, whose offset def_x * sign(x) depends on one sign.  Over
// the augmented input u = (x, y, dx, dy, 1, s_0, ..., s_{nb-1}) (s_b the sign
// of x at biprism b) every quantity of the paraxial chain is therefore a
// closed form the host composes in float64:
//   - each output coordinate: an affine row over u;
//   - each biprism's x and each aperture's (x, y): an affine row over the
//     signs decided before it (evaluated in chain order, so every sign is
//     known when a later row needs it);
//   - the per-ray pathlength terms (lens -(x^2 + y^2)/(2f); deflector and
//     biprism dx x + dy y with the incoming slopes, components.py:161-174,
//     476-482, 553-559): a quadratic form over u; its constant joins the
//     float64 uniform part.
// The kernel evaluates these in float32: one rounding per term instead of
// one per step, so deep chains with strong lenses (where step-by-step
// float32 loses up to ~1e-5 of the output scale to cancellation) stay at
// ~2e-7, and the rays run no step-dependent chain or per-component dispatch.
//
// Apertures.  A ray that an aperture blocks ((x-cx)^2 + (y-cy)^2 >= r^2 at
// the aperture) keeps its coordinates, is reported in the optional alive
// mask, and leaves the loss and every moment.
//
// Adjoint of loss = sum over alive rays of |(x, y)_out - target|^2 by moments.
// The loss gradient w.r.t. the output, l = 2 (x - tx, y - ty), reaches every
// step through the chain's LINEAR part, which is the same for every ray.
// Every per-step sum is therefore a fixed linear combination of a handful of
// per-model moments of the rays:
//   W[a][c] = sum_i l_a,i v_c,i     (v = input x, y, dx, dy, 1; a = x, y)
//   S_b[a]  = sum_i sign_b,i l_a,i  (one pair per biprism b)
// The host computes the combination coefficients in float64 (prefix maps,
// suffix maps and each biprism's propagated offset); the kernel accumulates
// the moments next to the forward pass (no reverse walk per ray) and the CTA
// that finishes a model's last tile contracts them, so one launch does the
// whole forward + adjoint.
#include <algorithm>
#include <cstring>
#include <vector>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(batch)

namespace tg {

struct BModel {
  int32_t op_off, n_steps, n_tiles, n_ev;  // n_ev: biprism + aperture events
  int64_t ray_off, n_rays;
  double pl_const, z_out;  // pl_const: float64 uniform pathlength plus the form's constant
  int64_t part_off;        // doubles: this model's first tile partial
  int32_t n_bip, n_mom;    // biprisms, moments (11 + 2 * n_bip)
  int64_t mom_off;         // doubles: this model's moments
  int64_t coef_off;        // doubles: per-step sum coefficients [n_steps][4][n_mom]
  int64_t rec_off;         // floats: this model's forward record
  int32_t rec_floats, ev_off;  // record length; first event (floats, in the record)
};

struct BTile {
  int32_t model, count;
  int64_t start;  // absolute ray index
  int32_t slot;   // tile index within its model: the partial's row
  int32_t pad;
};

struct BHeader {
  int32_t n_models, n_tiles, total_steps, tile_rays;
  int64_t models_off, tiles_off, ops_off, mom_model_off, rec_off, coef_off;  // byte offsets in the plan
  int64_t partial_doubles, moment_doubles;
};

// moment layout of one model
constexpr int kMomLoss = 10;  // W[a][c] at 5a + c (a = x, y), the loss at 10
constexpr int kMomBip = 11;   // S_b[a] at 11 + 2b + a
constexpr int kBatchMaxBip = 16;    // biprisms per model in the batched path
constexpr int kBatchMaxRec = 8192;  // floats per model record (staged in shared memory)
constexpr int kEvBiprism = 0, kEvAperture = 1;

// Forward record of one model (floats; every section 16-byte aligned), with
// D = 5 + nb and D4 = D rounded up to 4:
//   [0, 4D)        output map: column c of u as float4 (rows x, y, dx, dy)
//   [4D, 4D+16)    pathlength form over v: q[1..14] (q[0], q[15] unused)
//   next 8 nb      per biprism b: L_b[0..4] (its sign's linear term over v, 1)
//   next K4        K_bb' (b <= b', row-major upper triangle), padded to 4
//   events         per biprism / aperture in chain order: a header
//                  {kind, slot, r^2, cx, cy, 0, 0, 0}, the x row over u (D4),
//                  and for an aperture the y row (D4); an aperture's rows
//                  give x - cx and y - cy
struct RecLayout {
  int D, D4, q, l, k, ev, total;
};

__host__ __device__ inline RecLayout rec_layout(int nb, int n_bip_ev, int n_ap_ev) {
  RecLayout L;
  L.D = 5 + nb;
  L.D4 = (L.D + 3) & ~3;
  L.q = 4 * L.D;
  L.l = L.q + 16;
  L.k = L.l + 8 * nb;
  L.ev = L.k + ((nb * (nb + 1) / 2 + 3) & ~3);
  L.total = L.ev + n_bip_ev * (8 + L.D4) + n_ap_ev * (8 + 2 * L.D4);
  return L;
}

struct BatchIO {
  const float *x, *y, *dx, *dy;
  float *ox, *oy, *odx, *ody;
  double* opl;
  const float *tx, *ty;
  double* raw;
  uint8_t* alive;
  double* loss;
};

// 4-byte asynchronous global -> shared copy (zero-filled when src_bytes = 0)
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes)
               : "memory");
}

__device__ __forceinline__ float bt_warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sign of biprism b from the two bit masks (bit b of pos: +1, of neg: -1)
__device__ __forceinline__ float sign_of(uint32_t pos, uint32_t neg, int b) {
  return (float)((int)((pos >> b) & 1u) - (int)((neg >> b) & 1u));
}

// Models with more than four biprisms keep the first kRegBip sign moments in
// registers and warp-reduce the others per ray into shared memory.
constexpr int kRegBip = 4;

// Adjoint tail of one model, run by the CTA that stored the model's last tile
// partial (all threads of the CTA call it): the moments are the sum of the
// tile partials in tile order (each warp takes a moment, its lanes stride over
// tiles, a fixed shuffle tree combines them: deterministic); every per-step
// sum is then the float64 dot product of its coefficient row with them.
__device__ void batch_model_tail(const BModel& M, int model, const double* partial, const double* coef,
                                 double* moments_g, double* raw, double* loss, double* mo) {
  const int nm = M.n_mom;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const double* src = partial + M.part_off;
  for (int j = warp; j < nm; j += nwarps) {
    double a = 0.0;
    for (int t = lane; t < M.n_tiles; t += 32) a += __ldcg(src + (int64_t)t * nm + j);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) {
      mo[j] = a;
      moments_g[M.mom_off + j] = a;
    }
  }
  __syncthreads();
  const double* cf = coef + M.coef_off;
  for (int r = threadIdx.x; r < 4 * M.n_steps; r += blockDim.x) {
    const double* row = cf + (int64_t)r * nm;
    double acc = 0.0;
    for (int k = 0; k < nm; ++k) acc = fma(row[k], mo[k], acc);
    raw[(int64_t)M.op_off * 4 + r] = acc;
  }
  if (loss && threadIdx.x == 0) loss[model] = mo[kMomLoss];
}

// One tile of one model: every ray of the tile from start to finish (events,
// outputs, pathlength, stores, moments), then the tile's moments summed per
// warp into wacc.  NB = the model's biprism count when it is at most four:
// the signs live in registers and every loop over them is unrolled; NB = -1:
// any count, signs as bit masks with runtime loops.
template <int R, int NB>
__device__ __forceinline__ void batch_tile(const BatchIO& io, const BModel& M, const RecLayout& L,
                                           const float* srec, const float* pf, uint32_t pf_base,
                                           const BTile& T, int nf, bool adj, float* wacc) {
  constexpr int NS = NB > 0 ? NB : (NB < 0 ? kRegBip : 1);  // register sign slots
  const int nb = M.n_bip, nm = M.n_mom;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t t0 = T.start;
  float mw[11];
#pragma unroll
  for (int j = 0; j < 11; ++j) mw[j] = 0.f;
  float bsx[NS], bsy[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) bsx[j] = bsy[j] = 0.f;
  const int cnt = T.count;
  const int per = blockDim.x * R;
  // the next iteration's x, y, dx, dy (and targets) arrive by cp.async
  // (4-byte copies into this thread's own slots: no barrier) while this one
  // computes
  auto prefetch = [&](int it2, int st2) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int id = it2 + (int)threadIdx.x + k * (int)blockDim.x;
      const uint32_t sz = id < cnt ? 4u : 0u;
      const int i = id < cnt ? id : 0;
      const uint32_t b = pf_base + 4u * (uint32_t)((st2 * nf * R + k) * (int)blockDim.x + (int)threadIdx.x);
      const uint32_t fs = 4u * (uint32_t)(R * (int)blockDim.x);
      const int64_t g = t0 + i;
      cp_async4(b + 0 * fs, io.x + g, sz);
      cp_async4(b + 1 * fs, io.y + g, sz);
      cp_async4(b + 2 * fs, io.dx + g, sz);
      cp_async4(b + 3 * fs, io.dy + g, sz);
      if (adj) {
        cp_async4(b + 4 * fs, io.tx + g, sz);
        cp_async4(b + 5 * fs, io.ty + g, sz);
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  prefetch(0, 0);
  const float4* col = reinterpret_cast<const float4*>(srec);
  const float* q = srec + L.q;
  for (int it = 0, st = 0; it < cnt; it += per, st ^= 1) {
    if (it + per < cnt) prefetch(it + per, st ^ 1);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");
    const int fsf = R * (int)blockDim.x;
    // one ray at a time from start to finish: only its state is live, and
    // the record's coefficients are re-read from shared memory per ray
#pragma unroll 1
    for (int k = 0; k < R; ++k) {
      const int idx = it + (int)threadIdx.x + k * (int)blockDim.x;
      const float* pb = pf + (st * nf * R + k) * (int)blockDim.x + (int)threadIdx.x;
      const float v[4] = {pb[0], pb[fsf], pb[2 * fsf], pb[3 * fsf]};
      float sg[NS];  // NB >= 0: sign of each biprism (0 until decided)
#pragma unroll
      for (int b = 0; b < NS; ++b) sg[b] = 0.f;
      uint32_t spos = 0u, sneg = 0u;  // NB < 0: bit b set when sign(x) > 0 / < 0
      bool alive = true;
      // row . u over the signs decided so far (rows hold 0 for later ones)
      // rows are 16-byte aligned and padded to a multiple of 4 floats: the
      // constant and the first three sign coefficients come in one vector
      auto dot = [&](const float* row, int nbs) {
        const float4 r = *reinterpret_cast<const float4*>(row);
        const float4 r2 = *reinterpret_cast<const float4*>(row + 4);  // const, s_0, s_1, s_2
        float acc = fmaf(r.w, v[3], fmaf(r.z, v[2], fmaf(r.y, v[1], fmaf(r.x, v[0], r2.x))));
        if (NB >= 0) {
#pragma unroll
          for (int b = 0; b < NS; ++b)
            if (b < NB) {
              const float cb = b == 0 ? r2.y : (b == 1 ? r2.z : (b == 2 ? r2.w : row[5 + b]));
              acc = fmaf(cb, sg[b], acc);
            }
        } else {
          for (int b = 0; b < nbs; ++b) acc = fmaf(row[5 + b], sign_of(spos, sneg, b), acc);
        }
        return acc;
      };
      // events in chain order: each biprism's sign, each aperture's test
      // (the aperture rows hold x - cx and y - cy)
      {
        const float* e = srec + M.ev_off;
        int nbs = 0;
        for (int qe = 0; qe < M.n_ev; ++qe) {
          const float4 h = *reinterpret_cast<const float4*>(e);  // kind, slot, r^2, cx
          const float* xr = e + 8;
          if (__float_as_int(h.x) == kEvBiprism) {
            const float xe = dot(xr, nbs);
            const float s = xe > 0.f ? 1.f : (xe < 0.f ? -1.f : 0.f);
            if (NB >= 0) {
#pragma unroll
              for (int b = 0; b < NS; ++b)
                if (b == nbs) sg[b] = s;
            } else {
              const uint32_t bit = 1u << (nbs & 31);
              spos |= s > 0.f ? bit : 0u;
              sneg |= s < 0.f ? bit : 0u;
            }
            ++nbs;
            e += 8 + L.D4;
          } else {
            const float ex = dot(xr, nbs), ey = dot(xr + L.D4, nbs);
            alive = alive && (fmaf(ex, ex, ey * ey) < h.z);
            e += 8 + 2 * L.D4;
          }
        }
      }
      // outputs (the output map's columns over u) and the pathlength form:
      // q[1..4] linear in (x, y, dx, dy); q[5..8] x * (x, y, dx, dy);
      // q[9..11] y * (y, dx, dy); q[12..13] dx * (dx, dy); q[14] dy * dy
      const float4 c4 = col[4];
      float a0 = c4.x, a1 = c4.y, a2 = c4.z, a3 = c4.w;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float4 cc = col[c];
        a0 = fmaf(cc.x, v[c], a0); a1 = fmaf(cc.y, v[c], a1);
        a2 = fmaf(cc.z, v[c], a2); a3 = fmaf(cc.w, v[c], a3);
      }
      float p;
      {
        const float4 qa = *reinterpret_cast<const float4*>(q), qb = *reinterpret_cast<const float4*>(q + 4);
        const float4 qc = *reinterpret_cast<const float4*>(q + 8), qd = *reinterpret_cast<const float4*>(q + 12);
        const float t0q = fmaf(v[3], qc.x, fmaf(v[2], qb.w, fmaf(v[1], qb.z, fmaf(v[0], qb.y, qa.y))));
        const float t1q = fmaf(v[3], qc.w, fmaf(v[2], qc.z, fmaf(v[1], qc.y, qa.z)));
        const float t2q = fmaf(v[3], qd.y, fmaf(v[2], qd.x, qa.w));
        const float t3q = fmaf(v[3], qd.z, qb.x);
        p = fmaf(v[0], t0q, fmaf(v[1], t1q, fmaf(v[2], t2q, v[3] * t3q)));
      }
      auto sign_term = [&](int b, float s) {
        const float4 cb = col[5 + b];
        a0 = fmaf(cb.x, s, a0); a1 = fmaf(cb.y, s, a1); a2 = fmaf(cb.z, s, a2); a3 = fmaf(cb.w, s, a3);
        const float* lb = srec + L.l + 8 * b;
        const float4 l4 = *reinterpret_cast<const float4*>(lb);
        const float l5 = reinterpret_cast<const float4*>(lb)[1].x;
        float lin = fmaf(l4.x, v[0], fmaf(l4.y, v[1], fmaf(l4.z, v[2], fmaf(l4.w, v[3], l5))));
        const float* kb = srec + L.k + b * nb - (b * (b - 1)) / 2;  // K_bb' for b' >= b
        if (NB >= 0) {
#pragma unroll
          for (int b2 = 0; b2 < NS; ++b2)
            if (b2 >= b && b2 < NB) lin = fmaf(kb[b2 - b], sg[b2], lin);
        } else {
          for (int b2 = b; b2 < nb; ++b2) lin = fmaf(kb[b2 - b], sign_of(spos, sneg, b2), lin);
        }
        p = fmaf(s, lin, p);
      };
      if (NB >= 0) {
#pragma unroll
        for (int b = 0; b < NS; ++b)
          if (b < NB) sign_term(b, sg[b]);
      } else {
        for (int b = 0; b < nb; ++b) sign_term(b, sign_of(spos, sneg, b));
      }
      const bool inr = idx < cnt;
      if (inr) {
        const int64_t i = t0 + idx;
        io.ox[i] = a0;
        io.oy[i] = a1;
        io.odx[i] = a2;
        io.ody[i] = a3;
        if (io.opl) io.opl[i] = M.pl_const + (double)p;
        if (io.alive) io.alive[i] = alive ? 1 : 0;
      }
      if (!adj) continue;
      const bool use = inr && alive;
      const float rx = use ? a0 - pb[4 * fsf] : 0.f, ry = use ? a1 - pb[5 * fsf] : 0.f;
      const float lx = 2.f * rx, ly = 2.f * ry;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        mw[c] = fmaf(lx, v[c], mw[c]);
        mw[5 + c] = fmaf(ly, v[c], mw[5 + c]);
      }
      mw[4] += lx;
      mw[9] += ly;
      mw[kMomLoss] = fmaf(rx, rx, fmaf(ry, ry, mw[kMomLoss]));
      // biprism sign moments: registers for the first NS, warp sums beyond
#pragma unroll
      for (int b2 = 0; b2 < NS; ++b2) {
        if (NB >= 0 ? b2 < NB : b2 < nb) {
          const float s = NB >= 0 ? sg[b2] : sign_of(spos, sneg, b2);
          bsx[b2] = fmaf(s, lx, bsx[b2]);
          bsy[b2] = fmaf(s, ly, bsy[b2]);
        }
      }
      if (NB < 0) {
        for (int b2 = NS; b2 < nb; ++b2) {
          const float s = sign_of(spos, sneg, b2);
          const float sx = bt_warp_sum(s * lx), sy = bt_warp_sum(s * ly);
          if (lane == 0) {
            wacc[warp * nm + kMomBip + 2 * b2] += sx;
            wacc[warp * nm + kMomBip + 1 + 2 * b2] += sy;
          }
        }
      }
    }
  }
  if (adj) {
#pragma unroll
    for (int j = 0; j < 11; ++j) {
      const float s = bt_warp_sum(mw[j]);
      if (lane == 0) wacc[warp * nm + j] += s;
    }
#pragma unroll
    for (int b2 = 0; b2 < NS; ++b2) {
      if (NB >= 0 ? b2 < NB : b2 < nb) {
        const float sx = bt_warp_sum(bsx[b2]), sy = bt_warp_sum(bsy[b2]);
        if (lane == 0) {
          wacc[warp * nm + kMomBip + 2 * b2] += sx;
          wacc[warp * nm + kMomBip + 1 + 2 * b2] += sy;
        }
      }
    }
  }
}

template <int R>
__global__ void __launch_bounds__(512, (R == 4 ? 1 : 2))  // R = 1, 2: <= 64 registers (32 warps per SM)
k_batch(const uint8_t* __restrict__ plan, const __grid_constant__ BatchIO io,
        int32_t* __restrict__ counter, int32_t* __restrict__ done, double* __restrict__ partial,
        double* __restrict__ moments, int pf_off, int rec_smem_off) {
  // dynamic shared memory: [warps][n_mom] per-warp float32 moments of the tile
  // (reused by the model's adjoint tail for the float64 moments), the model
  // record, then the input stages [2][fields][R][blockDim] float32 (x, y,
  // dx, dy, and with targets tx, ty)
  extern __shared__ __align__(16) float wacc[];
  float* pf = wacc + pf_off;
  float* srec = wacc + rec_smem_off;
  const uint32_t pf_base = (uint32_t)__cvta_generic_to_shared(pf);
  __shared__ int s_last;
  __shared__ int s_tile;
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const BModel* models = reinterpret_cast<const BModel*>(plan + H.models_off);
  const BTile* tiles = reinterpret_cast<const BTile*>(plan + H.tiles_off);
  const float* recs = reinterpret_cast<const float*>(plan + H.rec_off);
  const double* coef = reinterpret_cast<const double*>(plan + H.coef_off);
  const bool adj = io.tx != nullptr;
  const int nf = adj ? 6 : 4;  // staged fields
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= H.n_tiles) break;
    const BTile T = tiles[t];
    if (T.model < 0 || T.model >= H.n_models) {  // corrupt plan: flag and skip
      if (threadIdx.x == 0) atomicOr(&g_tg_err, TG_EW_TABLE);
      __syncthreads();
      continue;
    }
    const BModel M = models[T.model];
    if (T.slot < 0 || T.slot >= M.n_tiles || M.n_bip < 0 || M.n_bip > kBatchMaxBip || M.rec_floats < 0 ||
        M.rec_floats > kBatchMaxRec || (M.rec_floats & 3) || M.ev_off < 0 || M.ev_off > M.rec_floats) {
      if (threadIdx.x == 0) atomicOr(&g_tg_err, TG_EW_TABLE);  // corrupt plan: flag and skip
      __syncthreads();
      continue;
    }
    const int nm = M.n_mom, nb = M.n_bip;
    const RecLayout L = rec_layout(nb, 0, 0);
    {
      const float4* src = reinterpret_cast<const float4*>(recs + M.rec_off);
      float4* dst = reinterpret_cast<float4*>(srec);
      for (int i = threadIdx.x; i < (M.rec_floats >> 2); i += blockDim.x) dst[i] = __ldg(src + i);
    }
    if (adj)
      for (int i = threadIdx.x; i < nwarps * nm; i += blockDim.x) wacc[i] = 0.f;
    __syncthreads();
    switch (nb) {  // signs as registers in fully unrolled loops for up to four biprisms
      case 0: batch_tile<R, 0>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
      case 1: batch_tile<R, 1>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
      case 2: batch_tile<R, 2>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
      case 3: batch_tile<R, 3>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
      case 4: batch_tile<R, 4>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
      default: batch_tile<R, -1>(io, M, L, srec, pf, pf_base, T, nf, adj, wacc); break;
    }
    __syncthreads();
    if (adj) {
      // warp 0 stores the tile partial and counts the tile; the CTA that
      // counts a model's last tile runs its adjoint tail (only warp 0 waits
      // for the fence, the other warps' ray stores are not ordered with it)
      if (warp == 0) {
        double* dst = partial + M.part_off + (int64_t)T.slot * nm;
        for (int i = lane; i < nm; i += 32) {
          double a = 0.0;
          for (int w = 0; w < nwarps; ++w) a += (double)wacc[w * nm + i];
          dst[i] = a;
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) s_last = atomicAdd(done + T.model, 1) == M.n_tiles - 1;
      }
      __syncthreads();
      if (s_last) {
        __threadfence();
        batch_model_tail(M, T.model, partial, coef, moments, io.raw, io.loss,
                         reinterpret_cast<double*>(wacc));
      }
    }
    __syncthreads();
  }
}

static int sm_count_batch() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  return cached;
}

static inline int64_t al16(int64_t v) { return (v + 15) & ~(int64_t)15; }
static inline int64_t al256(int64_t v) { return (v + 255) & ~(int64_t)255; }

static inline float int_bits_as_float(int v) {
  float f;
  std::memcpy(&f, &v, sizeof(f));
  return f;
}

// Host (float64): a model's forward record.  The state is carried as four
// affine rows over u = (x, y, dx, dy, 1, s_0, ..., s_{nb-1}) through the
// compiled steps; each pathlength term adds the symmetric product of two rows
// to the quadratic form Pi over u; events record the rows a biprism's sign or
// an aperture's test needs.  With rec == NULL only the sizes are reported.
static int batch_model_record(const tg_model& m, const Program& P, float* rec, double* pl_shift,
                              int* n_ev, int* rec_floats, int* ev_off) {
  const int nb = P.n_biprism, nc = P.n_steps / 2, D = 5 + nb;
  std::vector<double> row(4 * (size_t)D, 0.0), Pi((size_t)D * D, 0.0);
  for (int r = 0; r < 4; ++r) row[(size_t)r * D + r] = 1.0;
  auto R_ = [&](int r) { return &row[(size_t)r * D]; };
  auto add_prod = [&](double a, const double* p, const double* q) {  // Pi += a (p q^T + q p^T) / 2
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) Pi[(size_t)i * D + j] += 0.5 * a * (p[i] * q[j] + q[i] * p[j]);
  };
  struct Ev {
    int kind, slot;
    std::vector<double> x, y;
    double r2, cx, cy;
  };
  std::vector<Ev> evs;
  int nbip = 0, nap = 0;
  for (int i = 0; i < nc; ++i) {
    const double d = P.dstep[2 * i];
    for (int j = 0; j < D; ++j) {
      R_(0)[j] += d * R_(2)[j];
      R_(1)[j] += d * R_(3)[j];
    }
    const tg_component& c = m.components[i];
    const Op& op = P.op[2 * i + 1];
    switch (op.kind) {
      case OP_NOP:
        break;
      case OP_LENS: {
        const double f = c.p[0], h = 1.0 / (2.0 * f);
        add_prod(-h, R_(0), R_(0));
        add_prod(-h, R_(1), R_(1));
        for (int j = 0; j < D; ++j) {
          R_(2)[j] -= R_(0)[j] / f;
          R_(3)[j] -= R_(1)[j] / f;
        }
      } break;
      case OP_DEFLECT:
        add_prod(1.0, R_(2), R_(0));
        add_prod(1.0, R_(3), R_(1));
        R_(2)[4] += c.p[0];
        R_(3)[4] += c.p[1];
        break;
      case OP_BIPRISM: {
        evs.push_back(Ev{kEvBiprism, op.aux, std::vector<double>(R_(0), R_(0) + D), {}, 0.0, 0.0, 0.0});
        ++nbip;
        add_prod(1.0, R_(2), R_(0));
        add_prod(1.0, R_(3), R_(1));
        R_(2)[5 + op.aux] += c.p[0];
      } break;
      case OP_APERTURE:
        evs.push_back(Ev{kEvAperture, nap, std::vector<double>(R_(0), R_(0) + D),
                         std::vector<double>(R_(1), R_(1) + D), c.p[0] * c.p[0], c.p[1], c.p[2]});
        ++nap;
        break;
      case OP_SHIFT: {
        double cm[25];
        const int st = component_affine_f64(c, cm);
        if (st != TG_OK) return st;
        for (int r = 0; r < 4; ++r) R_(r)[4] += cm[5 * r + 4];
      } break;
      case OP_ROTATE: {
        const double a = c.p[0] * (M_PI / 180.0), ca = std::cos(a), sa = std::sin(a);
        for (int j = 0; j < D; ++j) {
          const double x = R_(0)[j], y = R_(1)[j], dx = R_(2)[j], dy = R_(3)[j];
          R_(0)[j] = x * ca - y * sa;
          R_(1)[j] = x * sa + y * ca;
          R_(2)[j] = dx * ca - dy * sa;
          R_(3)[j] = dx * sa + dy * ca;
        }
      } break;
      default:
        return TG_ERR_UNSUPPORTED;
    }
  }
  const RecLayout L = rec_layout(nb, nbip, nap);
  *n_ev = nbip + nap;
  *rec_floats = L.total;
  *ev_off = L.ev;
  auto pi = [&](int i, int j) { return Pi[(size_t)i * D + j]; };
  *pl_shift = pi(4, 4);  // the form's constant joins the float64 uniform part
  if (!rec) return TG_OK;
  std::memset(rec, 0, sizeof(float) * (size_t)L.total);
  for (int c = 0; c < D; ++c)
    for (int r = 0; r < 4; ++r) rec[4 * c + r] = (float)R_(r)[c];
  float* q = rec + L.q;
  for (int i = 0; i < 4; ++i) q[1 + i] = (float)(2.0 * pi(i, 4));  // linear in (x, y, dx, dy)
  int qi = 5;  // quadratic, row by row of the upper triangle
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j) q[qi++] = (float)((i == j ? 1.0 : 2.0) * pi(i, j));
  for (int b = 0; b < nb; ++b) {
    float* lb = rec + L.l + 8 * b;
    for (int c = 0; c < 5; ++c) lb[c] = (float)(2.0 * pi(5 + b, c));
    float* kb = rec + L.k + b * nb - (b * (b - 1)) / 2;
    for (int b2 = b; b2 < nb; ++b2) kb[b2 - b] = (float)((b2 == b ? 1.0 : 2.0) * pi(5 + b, 5 + b2));
  }
  float* e = rec + L.ev;
  for (const Ev& ev : evs) {
    e[0] = int_bits_as_float(ev.kind);
    e[1] = int_bits_as_float(ev.slot);
    e[2] = (float)ev.r2;
    e[3] = (float)ev.cx;
    e[4] = (float)ev.cy;
    for (int j = 0; j < D; ++j) e[8 + j] = (float)(ev.x[j] - (j == 4 ? ev.cx : 0.0));
    if (ev.kind == kEvAperture)
      for (int j = 0; j < D; ++j) e[8 + L.D4 + j] = (float)(ev.y[j] - (j == 4 ? ev.cy : 0.0));
    e += 8 + (ev.kind == kEvAperture ? 2 : 1) * L.D4;
  }
  return TG_OK;
}

// Host (float64): a model's per-step sum coefficients.
//   T_s      affine 5x5 of step s (a biprism is the identity here),
//   P_s      prefix T_s ... T_0 (state after step s, without biprism offsets),
//   G_s      suffix T_{n-1} ... T_{s+1} (linear part, rows x and y used),
//   phi_s,b  the change of the state after step s caused by biprism b's
//            offset def_b * (unit sign), for b at or before s.
// Per-step sums over alive
// rays (the quantities of tg_trace_vjp), with l_a = 2 (out_a - target_a):
//   propagator d, lens f, rotator angle (rad): dT_s/dp = Q_s T_s (free, lens:
//     Q_s T_s = dT_s/dp because Q_s^2 = 0; rotation: Q_s is its generator),
//     so sum_i l_i . G_s Q_s u_s,i with u_s = P_s v + sum_b sign_b phi_s,b:
//     coefficients (G_s Q_s P_s)[a][c] on W[a][c], (G_s Q_s phi_s,b)[a] on S_b[a];
//   shift (x, y, dx, dy), deflector (def_x, def_y): G_s[a][j] on W[a][4];
//   biprism b (def_x): G_s[a][2] on S_b[a].
static int batch_model_coefs(const tg_model& m, const Program& P, double* coef, int nm) {
  const int ns = P.n_steps, nc = ns / 2, nb = P.n_biprism;
  std::vector<double> T(25 * (size_t)ns), Pf(25 * (size_t)ns), G(25 * (size_t)ns);
  std::vector<double> phi(4 * (size_t)ns * (nb > 0 ? nb : 1), 0.0);
  std::vector<int> bip(ns, -1);
  std::vector<double> bdef(nb > 0 ? nb : 1, 0.0);
  for (int i = 0; i < nc; ++i) {
    double* F = &T[25 * (size_t)(2 * i)];
    std::memset(F, 0, 25 * sizeof(double));
    for (int k = 0; k < 5; ++k) F[6 * k] = 1.0;
    F[2] = P.dstep[2 * i];   // [0,2]
    F[8] = P.dstep[2 * i];   // [1,3]
    int st = component_affine_f64(m.components[i], &T[25 * (size_t)(2 * i + 1)]);
    if (st != TG_OK) return st;
    if (P.op[2 * i + 1].kind == OP_BIPRISM) {
      bip[2 * i + 1] = P.op[2 * i + 1].aux;
      bdef[P.op[2 * i + 1].aux] = m.components[i].p[0];
    }
  }
  auto mul5 = [](const double* a, const double* b, double* out) {
    double t[25];
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j) {
        double s = 0.0;
        for (int k = 0; k < 5; ++k) s += a[5 * i + k] * b[5 * k + j];
        t[5 * i + j] = s;
      }
    std::memcpy(out, t, sizeof(t));
  };
  for (int s = 0; s < ns; ++s) {  // prefixes and propagated biprism offsets
    if (s == 0) std::memcpy(&Pf[0], &T[0], 25 * sizeof(double));
    else mul5(&T[25 * (size_t)s], &Pf[25 * (size_t)(s - 1)], &Pf[25 * (size_t)s]);
    for (int b = 0; b < nb; ++b) {
      double* cur = &phi[4 * ((size_t)s * nb + b)];
      if (s > 0) {
        const double* prev = &phi[4 * ((size_t)(s - 1) * nb + b)];
        const double* Ts = &T[25 * (size_t)s];
        for (int r = 0; r < 4; ++r) {
          double v = 0.0;
          for (int k = 0; k < 4; ++k) v += Ts[5 * r + k] * prev[k];
          cur[r] = v;
        }
      }
      if (bip[s] == b) cur[2] += bdef[b];
    }
  }
  for (int s = ns - 1; s >= 0; --s) {  // suffixes
    double* g = &G[25 * (size_t)s];
    if (s == ns - 1) {
      std::memset(g, 0, 25 * sizeof(double));
      for (int k = 0; k < 5; ++k) g[6 * k] = 1.0;
    } else {
      mul5(&G[25 * (size_t)(s + 1)], &T[25 * (size_t)(s + 1)], g);
    }
  }
  std::memset(coef, 0, sizeof(double) * (size_t)ns * 4 * nm);
  for (int s = 0; s < ns; ++s) {
    const double* g = &G[25 * (size_t)s];
    const double* ps = &Pf[25 * (size_t)s];
    double* row = coef + (size_t)s * 4 * nm;
    const int kind = P.op[s].kind;
    double Q[25];
    bool bil = true;
    std::memset(Q, 0, sizeof(Q));
    if (kind == OP_FREE) {
      Q[2] = 1.0; Q[8] = 1.0;  // [0,2], [1,3]
    } else if (kind == OP_LENS) {
      const double f = m.components[s / 2].p[0];
      Q[10] = 1.0 / (f * f); Q[16] = 1.0 / (f * f);  // [2,0], [3,1]
    } else if (kind == OP_ROTATE) {
      Q[1] = -1.0; Q[5] = 1.0; Q[13] = -1.0; Q[17] = 1.0;  // [0,1], [1,0], [2,3], [3,2]
    } else {
      bil = false;
    }
    if (bil) {
      double gq[2][5];
      for (int a = 0; a < 2; ++a)
        for (int j = 0; j < 5; ++j) {
          double v = 0.0;
          for (int k = 0; k < 5; ++k) v += g[5 * a + k] * Q[5 * k + j];
          gq[a][j] = v;
        }
      for (int a = 0; a < 2; ++a) {
        for (int c = 0; c < 5; ++c) {
          double v = 0.0;
          for (int j = 0; j < 5; ++j) v += gq[a][j] * ps[5 * j + c];
          row[5 * a + c] = v;
        }
        for (int b = 0; b < nb; ++b) {
          const double* ph = &phi[4 * ((size_t)s * nb + b)];
          double v = 0.0;
          for (int j = 0; j < 4; ++j) v += gq[a][j] * ph[j];
          row[kMomBip + 2 * b + a] = v;
        }
      }
    } else if (kind == OP_SHIFT) {
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 2; ++a) row[(size_t)j * nm + 5 * a + 4] = g[5 * a + j];
    } else if (kind == OP_DEFLECT) {
      for (int j = 0; j < 2; ++j)
        for (int a = 0; a < 2; ++a) row[(size_t)j * nm + 5 * a + 4] = g[5 * a + 2 + j];
    } else if (kind == OP_BIPRISM) {
      const int b = P.op[s].aux;
      for (int a = 0; a < 2; ++a) row[kMomBip + 2 * b + a] = g[5 * a + 2];
    }
  }
  return TG_OK;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_batch_plan(int32_t n_models, const tg_model* models, const int64_t* n_rays,
                             const double* z_in, int32_t tile_rays, void* plan, size_t plan_bytes,
                             tg_batch_info* info) {
  if (n_models < 0 || (n_models > 0 && (!models || !n_rays)) || tile_rays <= 0 || !info)
    return TG_ERR_INVALID;
  std::vector<BModel> bm(n_models);
  std::vector<BTile> bt;
  std::vector<Op> ops;
  std::vector<int32_t> mom_model;
  std::vector<float> recs;
  std::vector<double> coef;
  std::vector<int64_t> work;  // per tile: rays x (components + adjoint overhead)
  int64_t ray_off = 0, part_off = 0, mom_off = 0;
  int32_t max_steps = 0, max_mom = 11, max_rec = 4;
  const bool fill = plan != nullptr;
  for (int m = 0; m < n_models; ++m) {
    if (n_rays[m] < 0) return TG_ERR_INVALID;
    Program P;
    int st = compile_program(&models[m], false, z_in ? z_in[m] : 0.0, &P);
    if (st != TG_OK) return st;
    if (P.n_probe_ops || P.n_aber || P.dircos) return TG_ERR_UNSUPPORTED;
    if (P.n_biprism > kBatchMaxBip) return TG_ERR_TOO_LARGE;
    double pl_shift = 0.0;
    int n_ev = 0, rec_floats = 0, ev_off = 0;
    st = batch_model_record(models[m], P, nullptr, &pl_shift, &n_ev, &rec_floats, &ev_off);
    if (st != TG_OK) return st;
    if (rec_floats > kBatchMaxRec) return TG_ERR_TOO_LARGE;
    BModel& M = bm[m];
    std::memset(&M, 0, sizeof(M));
    M.op_off = (int32_t)ops.size();
    M.n_steps = P.n_steps;
    if (P.n_steps > max_steps) max_steps = P.n_steps;
    M.ray_off = ray_off;
    M.n_rays = n_rays[m];
    M.pl_const = P.pl_const + pl_shift;
    M.z_out = P.z_out;
    M.part_off = part_off;
    M.n_bip = P.n_biprism;
    M.n_mom = kMomBip + 2 * P.n_biprism;
    M.mom_off = mom_off;
    M.n_ev = n_ev;
    M.rec_off = (int64_t)recs.size();
    M.rec_floats = rec_floats;
    M.ev_off = ev_off;
    M.coef_off = (int64_t)coef.size();
    if (M.n_mom > max_mom) max_mom = M.n_mom;
    if (rec_floats > max_rec) max_rec = rec_floats;
    for (int s = 0; s < P.n_steps; ++s) ops.push_back(P.op[s]);
    for (int j = 0; j < M.n_mom; ++j) mom_model.push_back(m);
    recs.resize(recs.size() + (size_t)rec_floats, 0.f);
    coef.resize(coef.size() + (size_t)P.n_steps * 4 * M.n_mom, 0.0);
    if (fill) {
      st = batch_model_record(models[m], P, recs.data() + M.rec_off, &pl_shift, &n_ev, &rec_floats, &ev_off);
      if (st != TG_OK) return st;
      st = batch_model_coefs(models[m], P, coef.data() + M.coef_off, M.n_mom);
      if (st != TG_OK) return st;
    }
    int32_t nt = 0;
    // at least one tile per model: an empty model's tile (count 0) still runs
    // the model's adjoint tail, which then writes zero sums
    for (int64_t r = 0; r < n_rays[m] || nt == 0; r += tile_rays, ++nt) {
      BTile T;
      T.model = m;
      T.start = ray_off + r;
      T.count = (int32_t)((n_rays[m] - r) < tile_rays ? (n_rays[m] - r) : tile_rays);
      T.slot = nt;
      T.pad = 0;
      bt.push_back(T);
      work.push_back((int64_t)T.count * (P.n_steps / 2 + 2));
    }
    M.n_tiles = nt;
    part_off += (int64_t)nt * M.n_mom;
    mom_off += M.n_mom;
    ray_off += n_rays[m];
    if (bt.size() > 0x7fffffff || ops.size() > 0x7fffffff)
      return TG_ERR_TOO_LARGE;
  }
  {  // longest tiles first (the work counter hands them out in list order), so
     // the launch ends on small tiles; ties keep model order
    std::vector<int32_t> ord(bt.size());
    for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int32_t)i;
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return work[a] > work[b]; });
    std::vector<BTile> sorted(bt.size());
    for (size_t i = 0; i < ord.size(); ++i) sorted[i] = bt[ord[i]];
    bt.swap(sorted);
  }
  BHeader H;
  std::memset(&H, 0, sizeof(H));
  H.n_models = n_models;
  H.n_tiles = (int32_t)bt.size();
  H.total_steps = (int32_t)ops.size();
  H.tile_rays = tile_rays;
  int64_t off = al16(sizeof(BHeader));
  H.models_off = off; off = al16(off + (int64_t)sizeof(BModel) * n_models);
  H.tiles_off = off; off = al16(off + (int64_t)sizeof(BTile) * bt.size());
  H.ops_off = off; off = al16(off + (int64_t)sizeof(Op) * ops.size());
  H.mom_model_off = off; off = al16(off + (int64_t)sizeof(int32_t) * mom_model.size());
  H.rec_off = off; off = al16(off + (int64_t)sizeof(float) * recs.size());
  H.coef_off = off; off = al16(off + (int64_t)sizeof(double) * coef.size());
  H.partial_doubles = part_off;
  H.moment_doubles = mom_off;
  info->plan_bytes = (size_t)off;
  info->n_tiles = H.n_tiles;
  info->total_steps = H.total_steps;
  info->total_rays = ray_off;
  info->max_steps = max_steps;
  info->max_moments = max_mom;
  info->max_record_floats = max_rec;
  info->n_models = n_models;
  info->partial_doubles = part_off;
  info->moment_doubles = mom_off;
  // workspace: tile counter + per-model done counters | tile partials | moments
  info->workspace_bytes = (size_t)al256(4 + 4 * (int64_t)n_models) + (size_t)(part_off + mom_off) * sizeof(double);
  if (!plan) return TG_OK;  // size query
  if (plan_bytes < (size_t)off) return TG_ERR_WORKSPACE;
  uint8_t* p = reinterpret_cast<uint8_t*>(plan);
  std::memset(p, 0, (size_t)off);
  std::memcpy(p, &H, sizeof(H));
  if (n_models) std::memcpy(p + H.models_off, bm.data(), sizeof(BModel) * n_models);
  if (!bt.empty()) std::memcpy(p + H.tiles_off, bt.data(), sizeof(BTile) * bt.size());
  if (!ops.empty()) std::memcpy(p + H.ops_off, ops.data(), sizeof(Op) * ops.size());
  if (!mom_model.empty())
    std::memcpy(p + H.mom_model_off, mom_model.data(), sizeof(int32_t) * mom_model.size());
  if (!recs.empty()) std::memcpy(p + H.rec_off, recs.data(), sizeof(float) * recs.size());
  if (!coef.empty()) std::memcpy(p + H.coef_off, coef.data(), sizeof(double) * coef.size());
  return TG_OK;
}

extern "C" int tg_batch_run(const void* plan_dev, const tg_batch_info* info, const tg_batch_io* io,
                            int32_t block, int32_t rays_per_thread, void* workspace,
                            size_t ws_bytes, void* stream) {
  if (!plan_dev || !info || !io) return TG_ERR_INVALID;
  if (block != 128 && block != 256 && block != 512) return TG_ERR_INVALID;
  if (rays_per_thread != 1 && rays_per_thread != 2 && rays_per_thread != 4) return TG_ERR_INVALID;
  if (info->total_rays > 0 && (!io->x || !io->y || !io->dx || !io->dy || !io->out_x ||
                               !io->out_y || !io->out_dx || !io->out_dy))
    return TG_ERR_INVALID;
  const bool adj = io->target_x != nullptr;
  if (adj && (!io->target_y || !io->raw)) return TG_ERR_INVALID;
  if (!adj && io->loss) return TG_ERR_INVALID;  // the loss needs targets
  if (!workspace || ws_bytes < info->workspace_bytes) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int32_t* counter = reinterpret_cast<int32_t*>(workspace);
  int32_t* done = counter + 1;
  const size_t head = (size_t)al256(4 + 4 * (int64_t)info->n_models);
  double* partial = reinterpret_cast<double*>(reinterpret_cast<uint8_t*>(workspace) + head);
  double* moments = partial + info->partial_doubles;
  if (cudaMemsetAsync(counter, 0, 4 + 4 * (size_t)info->n_models, s) != cudaSuccess) return TG_ERR_CUDA;
  if (info->n_tiles == 0) return TG_OK;
  BatchIO A;
  A.x = io->x; A.y = io->y; A.dx = io->dx; A.dy = io->dy;
  A.ox = io->out_x; A.oy = io->out_y; A.odx = io->out_dx; A.ody = io->out_dy;
  A.opl = io->out_pathlength;
  A.tx = io->target_x; A.ty = io->target_y;
  A.raw = io->raw;
  A.alive = io->out_alive;
  A.loss = io->loss;
  const uint8_t* plan = reinterpret_cast<const uint8_t*>(plan_dev);
  // dynamic shared memory: per-warp float32 moments (warps x max moments),
  // reused by the adjoint tail for the float64 moments; the largest model
  // record; then the input stages
  const size_t mom = (size_t)(info->max_moments > 0 ? info->max_moments : 11);
  if (info->max_record_floats < 0 || info->max_record_floats > kBatchMaxRec) return TG_ERR_INVALID;
  size_t dyn = (size_t)(block / 32) * mom * sizeof(float);
  const size_t tail = adj ? ((mom + 1) & ~(size_t)1) * sizeof(double) : 0;
  if (tail > dyn) dyn = tail;
  dyn = (dyn + 15) & ~(size_t)15;
  const int rec_smem_off = (int)(dyn / sizeof(float));
  dyn += ((size_t)info->max_record_floats * sizeof(float) + 15) & ~(size_t)15;
  const int pf_off = (int)(dyn / sizeof(float));
  dyn += (size_t)2 * (adj ? 6 : 4) * rays_per_thread * block * sizeof(float);
  if (dyn > 200 * 1024) return TG_ERR_TOO_LARGE;
  if (rays_per_thread == 1) cudaFuncSetAttribute(k_batch<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  else if (rays_per_thread == 2) cudaFuncSetAttribute(k_batch<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  else cudaFuncSetAttribute(k_batch<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  int per_sm = 1;
  if (rays_per_thread == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<1>, block, dyn);
  else if (rays_per_thread == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<2>, block, dyn);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<4>, block, dyn);
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count_batch() * per_sm;
  if (grid > info->n_tiles) grid = info->n_tiles;
  if (rays_per_thread == 1)
    k_batch<1><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off, rec_smem_off);
  else if (rays_per_thread == 2)
    k_batch<2><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off, rec_smem_off);
  else
    k_batch<4><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off, rec_smem_off);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

// One call for callers that do not keep a plan: pack the models on the host,
// copy the plan into the front of the caller's workspace (a synchronous
// staging copy from pageable memory, so this entry point is not for graph
// capture: tg_batch_plan + tg_batch_run are) and run with the launch shape
// measured best on GB300 (tiles of 4,096 rays, 256 threads x 2 rays).
namespace tg {
constexpr int32_t kDefTile = 4096, kDefBlock = 256, kDefRpt = 2;
}

extern "C" size_t tg_batched_trace_workspace(int32_t n_models, const tg_model* models,
                                             const int64_t* n_rays, const double* z_in) {
  tg_batch_info info;
  if (tg_batch_plan(n_models, models, n_rays, z_in, kDefTile, nullptr, 0, &info) != TG_OK) return 0;
  return (size_t)al256((int64_t)info.plan_bytes) + info.workspace_bytes;
}

extern "C" int tg_batched_trace(int32_t n_models, const tg_model* models, const int64_t* n_rays,
                                const double* z_in, const tg_batch_io* io, void* workspace,
                                size_t ws_bytes, void* stream) {
  tg_batch_info info;
  int st = tg_batch_plan(n_models, models, n_rays, z_in, kDefTile, nullptr, 0, &info);
  if (st != TG_OK) return st;
  const size_t head = (size_t)al256((int64_t)info.plan_bytes);
  if (!workspace || ws_bytes < head + info.workspace_bytes) return TG_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255) != 0) return TG_ERR_ALIGN;
  std::vector<uint8_t> host(info.plan_bytes);
  st = tg_batch_plan(n_models, models, n_rays, z_in, kDefTile, host.data(), host.size(), &info);
  if (st != TG_OK) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(workspace, host.data(), host.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return TG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return TG_ERR_CUDA;  // the host plan goes out of scope
  return tg_batch_run(workspace, &info, io, kDefBlock, kDefRpt, reinterpret_cast<uint8_t*>(workspace) + head,
                      ws_bytes - head, stream);
}
