// batch.cu - many independent models with uneven component and ray counts in
// ONE persistent launch over a packed model table (forward + adjoint).
//
// The reference runs each model separately (run.py:85-116 per model, jax.grad
// per model); here the host packs every model's compiled steps, a per-model
// header and a tile list into one device buffer (the plan).  A persistent
// grid pulls tiles (a model and a contiguous run of its rays) from an atomic
// work counter, stages that model's steps in shared memory, traces the rays
// forward and writes the outputs.  Per-tile partials are reduced per model in
// a fixed order, so the results do not depend on which CTA took which tile.
//
// Adjoint of loss = sum |(x, y)_out - target|^2 by moments.  The loss gradient
// w.r.t. the output, l = 2 (x - tx, y - ty), reaches every step through the
// LINEAR part of the chain, which is the same for every ray (a biprism's
// sign(x) only moves the affine offset).  Every per-step sum therefore follows
// exactly from a handful of per-model moments of the rays:
//   W[a][c] = sum_i l_a,i v_c,i     (v = input x, y, dx, dy, 1; a = x, y)
//   S_b[a]  = sum_i sign_b,i l_a,i  (one pair per biprism b)
// k_batch accumulates the moments next to the forward pass (no reverse walk
// per ray); the CTA that finishes a model's last tile reduces its moments and
// turns them into the per-step sums with 5x5 algebra (batch_model_tail), so
// one launch does the whole forward + adjoint.
#include <algorithm>
#include <cstring>
#include <vector>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(batch)

namespace tg {

struct BModel {
  int32_t op_off, n_steps, n_tiles, pad;
  int64_t ray_off, n_rays;
  double pl_const, z_out;
  int64_t part_off;  // doubles: this model's first tile partial
  int32_t n_bip, n_mom;  // biprisms, moments (10 + 2 * n_bip)
  int64_t mom_off;       // doubles: this model's moments
};

struct BTile {
  int32_t model, count;
  int64_t start;  // absolute ray index
  int32_t slot;   // tile index within its model: the partial's row
  int32_t pad;
};

struct BHeader {
  int32_t n_models, n_tiles, total_steps, tile_rays;
  int64_t models_off, tiles_off, ops_off, mom_model_off;  // byte offsets in the plan
  int64_t partial_doubles, moment_doubles;
};

struct BatchIO {
  const float *x, *y, *dx, *dy;
  float *ox, *oy, *odx, *ody;
  double* opl;
  const float *tx, *ty;
  double* raw;
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

// One component with the free-space step in front of it (the compiled
// program always alternates the two), 32 bytes: two float4 broadcasts from
// shared memory per component and one kind test for all of a thread's rays.
struct FOp {
  int32_t kind;  // component op (OP_NOP for a plane / detector)
  int32_t aux;   // OP_BIPRISM: sign slot
  float d;       // propagation distance before the component
  float c[5];
};
static_assert(sizeof(FOp) == 32, "FOp is two float4");

// Biprism sign moments kept in registers for the first kRegBip biprisms of a
// model; any further ones are warp-reduced per iteration into shared memory.
constexpr int kRegBip = 4;

// Entry (i, j) of the 5x5 step matrix of one compiled step (linear part +
// non-biprism offsets, in the float32 values the forward pass used; 0 outside
// the 5x5 range).  A biprism's offset enters through its sign moment; the
// other kinds are the identity.
__device__ __forceinline__ float t_entry(const Op& op, int i, int j) {
  if (i > 4 || j > 4) return 0.f;
  float v = (i == j) ? 1.f : 0.f;
  switch (op.kind) {
    case OP_FREE: if ((i == 0 && j == 2) || (i == 1 && j == 3)) v = op.c[0]; break;
    case OP_LENS: if ((i == 2 && j == 0) || (i == 3 && j == 1)) v = -op.c[0]; break;
    case OP_SHIFT:  // register selects, not a dynamic index into op.c
      if (j == 4 && i < 4) v = i == 0 ? op.c[0] : (i == 1 ? op.c[1] : (i == 2 ? op.c[2] : op.c[3]));
      break;
    case OP_DEFLECT: if (j == 4 && (i == 2 || i == 3)) v = i == 2 ? op.c[0] : op.c[1]; break;
    case OP_ROTATE:
      if (i < 4 && j < 4 && (i >> 1) == (j >> 1)) {
        const int ii = i & 1, jj = j & 1;
        v = (ii == jj) ? op.c[0] : (ii == 0 ? -op.c[1] : op.c[1]);
      }
      break;
    default: break;
  }
  return v;
}

// Step s of the compiled program (propagator, component, propagator, ...)
// rebuilt from the fused per-component records staged in shared memory.
__device__ __forceinline__ Op fused_step(const FOp* f, int s) {
  Op o;
  const FOp& c = f[s >> 1];
  if ((s & 1) == 0) {
    o.kind = OP_FREE;
    o.aux = 0;
    o.c[0] = c.d;
    for (int j = 1; j < 6; ++j) o.c[j] = 0.f;
  } else {
    o.kind = c.kind;
    o.aux = c.aux;
    for (int j = 0; j < 5; ++j) o.c[j] = c.c[j];
    o.c[5] = 0.f;
  }
  return o;
}

// Adjoint tail of one model, run by the CTA that stored the model's last tile
// partial (all threads of the CTA call it).  Per-step sums, the quantities of
// the generic adjoint, follow from the moments:
//  1. moments = sum of the tile partials in tile order (each warp takes a
//     moment; its lanes stride over tiles; a fixed shuffle tree combines them,
//     so the result is deterministic);
//  2. warp 0 walks the chain backwards for G_s = linear part of
//     (T_{ns-1} ... T_{s+1}) and warp 1 walks it forwards for the first four
//     rows of the prefix C_s and the moment-weighted biprism offsets E_s
//     (E_{s,a} = sum_b S_b[a] (effect at step s of biprism b's offset)); the
//     5x5 products run in float32, the precision of the traced rays;
//  3. every thread contracts steps with the moments in float64:
//     sum_a (G_s Q C_s)[a] . W[a] + (G_s Q E_{s,a})[a].
constexpr int kStepFloats = 16 + 20 + 8;  // G_s, C_s rows 0..3, E_s (a = x, y)

__device__ void batch_model_tail(const BModel& M, const FOp* fops, const double* partial,
                                 double* moments_g, double* raw, float* smem) {
  const int nm = M.n_mom, ns = M.n_steps;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  double* mo = reinterpret_cast<double*>(smem);                // [nm]
  float* st = reinterpret_cast<float*>(mo + ((nm + 1) & ~1));  // [ns][kStepFloats]
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
  // The chain walks keep one matrix element per lane and combine them with
  // shuffles (same multiply-add order as a row-by-column product).
  if (warp == 0) {  // backward: G_s, lanes 0..15 own Rm[i][j], i = lane / 4, j = lane % 4
    const int i = lane >> 2, j = lane & 3;
    float rm = (i == j && lane < 16) ? 1.f : 0.f;
    for (int s = ns - 1; s >= 0; --s) {
      if (lane < 16) st[s * kStepFloats + lane] = rm;
      const Op op = fused_step(fops, s);
      float v = 0.f;
#pragma unroll
      for (int k = 0; k < 4; ++k) v = fmaf(__shfl_sync(0xffffffffu, rm, (i * 4 + k) & 31), t_entry(op, k, j), v);
      rm = v;
    }
  } else if (warp == 1) {  // forward: lanes 0..24 own Cm[i][j] (i = lane / 5); lanes 0..7 own E[a][ie]
    const int i = lane / 5, j = lane % 5;
    const int a = lane >> 2, ie = lane & 3;
    float cm = (i == j && lane < 25) ? 1.f : 0.f;
    float e = 0.f;
    for (int s = 0; s < ns; ++s) {
      const Op op = fused_step(fops, s);
      float v = 0.f;
#pragma unroll
      for (int k = 0; k < 5; ++k) v = fmaf(t_entry(op, i, k), __shfl_sync(0xffffffffu, cm, (k * 5 + j) & 31), v);
      float ve = 0.f;
#pragma unroll
      for (int k = 0; k < 4; ++k) ve = fmaf(t_entry(op, ie, k), __shfl_sync(0xffffffffu, e, (a * 4 + k) & 31), ve);
      cm = v;
      e = ve;
      if (op.kind == OP_BIPRISM && lane < 8 && ie == 2)  // this biprism's offset def * sign * e_dx, weighted by S_b
        e += (float)(op.c[0] * mo[10 + 2 * op.aux + a]);
      if (lane < 20) st[s * kStepFloats + 16 + lane] = cm;  // rows 0..3
      if (lane < 8) st[s * kStepFloats + 36 + lane] = e;
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const Op op = fused_step(fops, s);
    const float* Gs = st + s * kStepFloats;       // Gs[4*i+j]
    const float* Cs = Gs + 16;                    // Cs[5*i+j], rows 0..3
    const float* Es = Gs + 36;                    // Es[4*a+j]
    auto lin = [&](int j) { return (double)Gs[0 * 4 + j] * mo[4] + (double)Gs[1 * 4 + j] * mo[9]; };
    auto bil = [&](const float Q[4][4]) {
      double acc = 0.0;
      for (int a = 0; a < 2; ++a) {
        float GQ[4];
        for (int j = 0; j < 4; ++j) {
          float v = 0.f;
          for (int k = 0; k < 4; ++k) v = fmaf(Gs[a * 4 + k], Q[k][j], v);
          GQ[j] = v;
        }
        for (int c = 0; c < 5; ++c) {
          float v = 0.f;
          for (int j = 0; j < 4; ++j) v = fmaf(GQ[j], Cs[5 * j + c], v);
          acc += (double)v * mo[5 * a + c];
        }
        float v = 0.f;
        for (int j = 0; j < 4; ++j) v = fmaf(GQ[j], Es[4 * a + j], v);
        acc += (double)v;
      }
      return acc;
    };
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
    switch (op.kind) {
      case OP_FREE: {
        const float Q[4][4] = {{0, 0, 1, 0}, {0, 0, 0, 1}, {0, 0, 0, 0}, {0, 0, 0, 0}};
        r0 = bil(Q);
      } break;
      case OP_LENS: {
        const float k2 = op.c[0] * op.c[0];
        const float Q[4][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {k2, 0, 0, 0}, {0, k2, 0, 0}};
        r0 = bil(Q);
      } break;
      case OP_ROTATE: {
        const float Q[4][4] = {{0, -1, 0, 0}, {1, 0, 0, 0}, {0, 0, 0, -1}, {0, 0, 1, 0}};
        r0 = bil(Q);
      } break;
      case OP_SHIFT:
        r0 = lin(0); r1 = lin(1); r2 = lin(2); r3 = lin(3);
        break;
      case OP_DEFLECT:
        r0 = lin(2); r1 = lin(3);
        break;
      case OP_BIPRISM: {
        const int b = op.aux;
        r0 = (double)Gs[0 * 4 + 2] * mo[10 + 2 * b] + (double)Gs[1 * 4 + 2] * mo[11 + 2 * b];
      } break;
      default: break;
    }
    double* out = raw + (int64_t)(M.op_off + s) * 4;
    out[0] = r0; out[1] = r1; out[2] = r2; out[3] = r3;
  }
}

template <int R>
__global__ void __launch_bounds__(512, (R == 4 ? 1 : 2))  // R = 1, 2: <= 64 registers (32 warps per SM)
k_batch(const uint8_t* __restrict__ plan, const __grid_constant__ BatchIO io,
        int32_t* __restrict__ counter, int32_t* __restrict__ done, double* __restrict__ partial,
        double* __restrict__ moments, int pf_off) {
  // dynamic shared memory: [warps][n_mom] per-warp float32 moments of the tile,
  // reused by the model's adjoint tail (moments + per-step products)
  extern __shared__ __align__(16) float wacc[];
  float* pf = wacc + pf_off;  // input stages [2][4 fields][R][blockDim] float32
  const uint32_t pf_base = (uint32_t)__cvta_generic_to_shared(pf);
  __shared__ int s_last;
  __shared__ __align__(16) FOp sops[TG_MAX_COMPONENTS];
  __shared__ int s_tile;
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const BHeader H = *reinterpret_cast<const BHeader*>(plan);
  const BModel* models = reinterpret_cast<const BModel*>(plan + H.models_off);
  const BTile* tiles = reinterpret_cast<const BTile*>(plan + H.tiles_off);
  const Op* ops = reinterpret_cast<const Op*>(plan + H.ops_off);
  const bool adj = io.tx != nullptr;
  const int lane = threadIdx.x & 31;
  const float4* sf4 = reinterpret_cast<const float4*>(sops);
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
    if (T.slot < 0 || T.slot >= M.n_tiles) {  // corrupt plan: flag and skip
      if (threadIdx.x == 0) atomicOr(&g_tg_err, TG_EW_TABLE);
      __syncthreads();
      continue;
    }
    const int nc = M.n_steps >> 1, nm = M.n_mom, nb = M.n_bip;
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
      const Op fr = ops[M.op_off + 2 * i], co = ops[M.op_off + 2 * i + 1];
      FOp f;
      f.kind = co.kind;
      f.aux = co.aux;
      f.d = fr.c[0];
      for (int j = 0; j < 5; ++j) f.c[j] = co.c[j];
      if (fr.kind != OP_FREE) {  // the batched plan only holds uniform propagators
        atomicOr(&g_tg_err, TG_EW_TABLE);
        f.d = 0.f;
      }
      sops[i] = f;
    }
    if (adj)
      for (int i = threadIdx.x; i < nwarps * nm; i += blockDim.x) wacc[i] = 0.f;
    __syncthreads();
    // tile-local 32-bit indexing from per-tile base pointers
    const float* __restrict__ gx = io.x + T.start;
    const float* __restrict__ gy = io.y + T.start;
    const float* __restrict__ gdx = io.dx + T.start;
    const float* __restrict__ gdy = io.dy + T.start;
    float* __restrict__ ox = io.ox + T.start;
    float* __restrict__ oy = io.oy + T.start;
    float* __restrict__ odx = io.odx + T.start;
    float* __restrict__ ody = io.ody + T.start;
    double* __restrict__ opl = io.opl ? io.opl + T.start : nullptr;
    const float* __restrict__ gtx = adj ? io.tx + T.start : nullptr;
    const float* __restrict__ gty = adj ? io.ty + T.start : nullptr;
    float mw[10];
#pragma unroll
    for (int j = 0; j < 10; ++j) mw[j] = 0.f;
    float bsx[kRegBip], bsy[kRegBip];
#pragma unroll
    for (int j = 0; j < kRegBip; ++j) bsx[j] = bsy[j] = 0.f;
    const int cnt = T.count;
    const int per = blockDim.x * R;
    // the next iteration's x, y, dx, dy arrive by cp.async (4-byte copies into
    // this thread's own slots: no barrier) while this one computes; measured
    // on the 512-model sweep: forward 0.217 -> 0.200 ms, forward + adjoint
    // 0.250 -> 0.244 ms.  The targets, needed only after the chain, are plain
    // loads whose latency the chain hides, and the inputs are re-read from
    // the stage for the moments instead of being held in registers.
    auto prefetch = [&](int it2, int st2) {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int id = it2 + (int)threadIdx.x + k * (int)blockDim.x;
        const uint32_t sz = id < cnt ? 4u : 0u;
        const int i = id < cnt ? id : 0;
        const uint32_t b = pf_base + 4u * (uint32_t)((st2 * 4 * R + k) * (int)blockDim.x + (int)threadIdx.x);
        const uint32_t fs = 4u * (uint32_t)(R * (int)blockDim.x);
        cp_async4(b + 0 * fs, gx + i, sz);
        cp_async4(b + 1 * fs, gy + i, sz);
        cp_async4(b + 2 * fs, gdx + i, sz);
        cp_async4(b + 3 * fs, gdy + i, sz);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    prefetch(0, 0);
    for (int it = 0, st = 0; it < cnt; it += per, st ^= 1) {
      float x[R], y[R], dx[R], dy[R], pl[R], v0[R][4], tx[R], ty[R];
      uint32_t spos[R], sneg[R];  // biprism b: bit b set when sign(x) > 0 / < 0
      int idx[R];
      bool inr[R];
      if (it + per < cnt) prefetch(it + per, st ^ 1);
      else asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 1;" ::: "memory");
#pragma unroll
      for (int k = 0; k < R; ++k) {
        idx[k] = it + (int)threadIdx.x + k * (int)blockDim.x;  // coalesced per k
        inr[k] = idx[k] < cnt;
        const float* pb = pf + (st * 4 * R + k) * (int)blockDim.x + (int)threadIdx.x;
        const int fsf = R * (int)blockDim.x;
        x[k] = pb[0]; y[k] = pb[fsf]; dx[k] = pb[2 * fsf]; dy[k] = pb[3 * fsf];
        if (adj) {  // needed only after the chain: the chain hides the load latency
          const int i = inr[k] ? idx[k] : 0;
          tx[k] = gtx[i];
          ty[k] = gty[i];
        }
        pl[k] = 0.f;
        spos[k] = sneg[k] = 0u;
      }
      for (int s = 0; s < nc; ++s) {
        const float4 A = sf4[2 * s], B = sf4[2 * s + 1];  // {kind, aux, d, c0}, {c1..c4}
        const int kind = __float_as_int(A.x);
        const float d = A.z;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          x[k] = fmaf(dx[k], d, x[k]);
          y[k] = fmaf(dy[k], d, y[k]);
        }
        if (kind == OP_LENS) {
          const float k1 = A.w, h = B.x;
#pragma unroll
          for (int k = 0; k < R; ++k) {
            const float xx = x[k], yy = y[k];
            pl[k] -= (xx * xx + yy * yy) * h;
            dx[k] = fmaf(-xx, k1, dx[k]);
            dy[k] = fmaf(-yy, k1, dy[k]);
          }
        } else if (kind == OP_BIPRISM) {
          const uint32_t bit = 1u << __float_as_int(A.y);  // slot < 32
#pragma unroll
          for (int k = 0; k < R; ++k) {
            pl[k] += dx[k] * x[k] + dy[k] * y[k];
            const float sg = sgnf(x[k]);
            spos[k] |= sg > 0.f ? bit : 0u;
            sneg[k] |= sg < 0.f ? bit : 0u;
            dx[k] = fmaf(A.w, sg, dx[k]);
          }
        } else if (kind == OP_DEFLECT) {
#pragma unroll
          for (int k = 0; k < R; ++k) {
            pl[k] += dx[k] * x[k] + dy[k] * y[k];
            dx[k] += A.w;
            dy[k] += B.x;
          }
        } else if (kind == OP_SHIFT) {
#pragma unroll
          for (int k = 0; k < R; ++k) {
            x[k] += A.w; y[k] += B.x; dx[k] += B.y; dy[k] += B.z;
          }
        } else if (kind == OP_ROTATE) {
          const float c = A.w, sn = B.x;
#pragma unroll
          for (int k = 0; k < R; ++k) {
            const float xx = x[k], yy = y[k], ddx = dx[k], ddy = dy[k];
            x[k] = xx * c - yy * sn;
            y[k] = xx * sn + yy * c;
            dx[k] = ddx * c - ddy * sn;
            dy[k] = ddx * sn + ddy * c;
          }
        }
        // OP_APERTURE / OP_NOP: no change to the traced state (the batched
        // outputs carry no mask; the loss covers every ray)
      }
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (inr[k]) {
          const int i = idx[k];
          ox[i] = x[k];
          oy[i] = y[k];
          odx[i] = dx[k];
          ody[i] = dy[k];
          // the float64 add: add_f64_f32's integer rounding measured slower
          // in this register-bound kernel (0.318 vs 0.291 ms on the sweep)
          if (opl) opl[i] = M.pl_const + (double)pl[k];
        }
      }
      if (!adj) continue;
      float lx[R], ly[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        // inputs re-read from the stage (not held in registers through the chain)
        const float* pb = pf + (st * 4 * R + k) * (int)blockDim.x + (int)threadIdx.x;
        const int fsf = R * (int)blockDim.x;
        v0[k][0] = pb[0]; v0[k][1] = pb[fsf]; v0[k][2] = pb[2 * fsf]; v0[k][3] = pb[3 * fsf];
        lx[k] = inr[k] ? 2.f * (x[k] - tx[k]) : 0.f;
        ly[k] = inr[k] ? 2.f * (y[k] - ty[k]) : 0.f;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          mw[c] = fmaf(lx[k], v0[k][c], mw[c]);
          mw[5 + c] = fmaf(ly[k], v0[k][c], mw[5 + c]);
        }
        mw[4] += lx[k];
        mw[9] += ly[k];
      }
      // biprism sign moments: registers for the first kRegBip, warp sums beyond
#pragma unroll
      for (int b2 = 0; b2 < kRegBip; ++b2) {
        if (b2 < nb) {
#pragma unroll
          for (int k = 0; k < R; ++k) {
            const float sg = (spos[k] >> b2) & 1u ? 1.f : ((sneg[k] >> b2) & 1u ? -1.f : 0.f);
            bsx[b2] = fmaf(sg, lx[k], bsx[b2]);
            bsy[b2] = fmaf(sg, ly[k], bsy[b2]);
          }
        }
      }
      for (int b2 = kRegBip; b2 < nb; ++b2) {
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const float sg = (spos[k] >> b2) & 1u ? 1.f : ((sneg[k] >> b2) & 1u ? -1.f : 0.f);
          sx = fmaf(sg, lx[k], sx);
          sy = fmaf(sg, ly[k], sy);
        }
        sx = bt_warp_sum(sx);
        sy = bt_warp_sum(sy);
        if (lane == 0) {
          wacc[warp * nm + 10 + 2 * b2] += sx;
          wacc[warp * nm + 11 + 2 * b2] += sy;
        }
      }
    }
    if (adj) {
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const float v = bt_warp_sum(mw[j]);
        if (lane == 0) wacc[warp * nm + j] += v;
      }
#pragma unroll
      for (int b2 = 0; b2 < kRegBip; ++b2) {
        if (b2 < nb) {
          const float sx = bt_warp_sum(bsx[b2]), sy = bt_warp_sum(bsy[b2]);
          if (lane == 0) {
            wacc[warp * nm + 10 + 2 * b2] += sx;
            wacc[warp * nm + 11 + 2 * b2] += sy;
          }
        }
      }
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
        batch_model_tail(M, sops, partial, moments, io.raw, wacc);
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
  std::vector<int64_t> work;  // per tile: rays x (components + adjoint overhead)
  int64_t ray_off = 0, part_off = 0, mom_off = 0;
  int32_t max_steps = 0, max_mom = 10;
  for (int m = 0; m < n_models; ++m) {
    if (n_rays[m] < 0) return TG_ERR_INVALID;
    Program P;
    int st = compile_program(&models[m], false, z_in ? z_in[m] : 0.0, &P);
    if (st != TG_OK) return st;
    if (P.n_probe_ops || P.n_aber || P.dircos) return TG_ERR_UNSUPPORTED;
    BModel& M = bm[m];
    std::memset(&M, 0, sizeof(M));
    M.op_off = (int32_t)ops.size();
    M.n_steps = P.n_steps;
    if (P.n_steps > max_steps) max_steps = P.n_steps;
    M.ray_off = ray_off;
    M.n_rays = n_rays[m];
    M.pl_const = P.pl_const;
    M.z_out = P.z_out;
    M.part_off = part_off;
    M.n_bip = P.n_biprism;
    M.n_mom = 10 + 2 * P.n_biprism;
    M.mom_off = mom_off;
    if (M.n_mom > max_mom) max_mom = M.n_mom;
    for (int s = 0; s < P.n_steps; ++s) ops.push_back(P.op[s]);
    for (int j = 0; j < M.n_mom; ++j) mom_model.push_back(m);
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
    if (bt.size() > 0x7fffffff || ops.size() > 0x7fffffff) return TG_ERR_TOO_LARGE;
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
  H.partial_doubles = part_off;
  H.moment_doubles = mom_off;
  info->plan_bytes = (size_t)off;
  info->n_tiles = H.n_tiles;
  info->total_steps = H.total_steps;
  info->total_rays = ray_off;
  info->max_steps = max_steps;
  info->max_moments = max_mom;
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
  const uint8_t* plan = reinterpret_cast<const uint8_t*>(plan_dev);
  // dynamic shared memory: per-warp float32 moments (warps x max moments),
  // reused by the adjoint tail for the moments (float64) and the per-step products
  const size_t mom = (size_t)(info->max_moments > 0 ? info->max_moments : 10);
  const size_t tail = adj ? ((mom + 1) & ~(size_t)1) * sizeof(double) +
                                (size_t)(info->max_steps > 0 ? info->max_steps : 1) * kStepFloats * sizeof(float)
                          : 0;
  size_t dyn = (size_t)(block / 32) * mom * sizeof(float);
  if (tail > dyn) dyn = tail;
  dyn = (dyn + 15) & ~(size_t)15;
  const int pf_off = (int)(dyn / sizeof(float));
  dyn += (size_t)2 * 4 * rays_per_thread * block * sizeof(float);
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
  if (rays_per_thread == 1) k_batch<1><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off);
  else if (rays_per_thread == 2) k_batch<2><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off);
  else k_batch<4><<<grid, block, dyn, s>>>(plan, A, counter, done, partial, moments, pf_off);
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
