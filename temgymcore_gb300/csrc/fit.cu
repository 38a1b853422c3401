// fit.cu - on-device 4D-STEM calibration fit: loss + gradient w.r.t. the
// microscope parameters, and an Adam update, all reading the parameters
// from device memory so a whole optimisation step can be replayed as a CUDA
// graph without host round trips.
//
// Model (the reference composes it from components.py Scanner/Descanner/
// Lens/Detector and differentiates run_to_end with jax.grad, README.md:113-160):
//   bundle at z = 0 -> sample plane at z = defocus: Scanner(+s) and
//   Descanner(M s + off - s) with the probe's scan position s (ScanGrid map,
//   grid.py:155-182) -> Lens(f) at z = defocus + gap -> Detector at
//   z = defocus + camera_length.
// Parameters theta[21] = f, defocus, camera_length, scan rotation (deg),
// scan step, M (4x4 row-major: rows x, y, dx, dy; cols spx, spy, stx, sty).
// Loss = sum over probes and rays of |r_det - r_target|^2.
//
// k_stem_fit: one CTA per probe at a time; it derives the probe's scan
// geometry in float64, each thread runs the chain and its hand-derived
// adjoint for its rays in registers, and the CTA reduces the probe's sums.
// k_fit_reduce applies the chain rule through the scan geometry in float64
// and reduces in fixed order (deterministic); for a whole optimisation step
// (tg_stem_fit_step) the block that completes the last output also applies
// the Adam update, so a step is two launches.
#include <cstring>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(fit)

namespace tg {

constexpr int kFitThreads = 256;
constexpr int kFitOut = 22;  // loss + 21 gradients
constexpr int kRedChunks = 8;  // probe chunks per output in the reduction

struct FitArgs {
  int32_t n, rows, cols, n_probes;
  const float *x, *y, *dx, *dy;
  const float *tx, *ty;  // [n_probes][n]
  float *ox, *oy;        // forward mode outputs [n_probes][n] (may be NULL)
  const double* theta;
  double gap;
  double2* sp;           // [n_probes] scan position (x, y)
  double* psum;          // [n_probes][8] per-probe sums
  double2* rot;          // [1] cos, sin of the scan rotation (written by k_stem_fit)
  double* part;          // [kFitOut][kRedChunks] reduction partials
  int32_t* cnt;          // [kFitOut + 1] chunks counted per output, outputs done
                         // (zeroed by k_stem_fit before k_fit_reduce runs)
  int32_t forward_only;
  // Adam hand-off (tg_stem_fit_step): the block of k_fit_reduce that
  // completes the last output updates theta in place
  int32_t adam;
  double* theta_w;
  double *m, *v;
  int64_t* t;
  double lr, b1, b2, eps;
  const double* scale;
  const uint8_t* mask;
};

// b^n (n >= 0) by repeated squaring: the Adam bias corrections in at most 63
// float64 multiplies on the critical path instead of the pow library call.
__device__ __forceinline__ double powi(double b, int64_t n) {
  double r = 1.0;
  for (; n > 0; n >>= 1) {
    if (n & 1) r *= b;
    b *= b;
  }
  return r;
}

// One Adam update of parameter i < n (the step counter tt already advanced):
// gradients w.r.t. parameters normalised by their scale (Adam in relative
// units); mask: 1 = parameter is fitted.
__device__ __forceinline__ void adam_update(int i, double* theta, double g_raw, double* m, double* v,
                                            double lr, double b1, double b2, double eps,
                                            double c1, double c2, const double* scale,
                                            const uint8_t* mask) {
  if (mask && !mask[i]) return;
  const double sc = scale ? scale[i] : 1.0;
  const double g = g_raw * sc;
  m[i] = b1 * m[i] + (1.0 - b1) * g;
  v[i] = b2 * v[i] + (1.0 - b2) * g * g;
  const double mh = m[i] / c1, vh = v[i] / c2;
  theta[i] -= sc * lr * mh / (sqrt(vh) + eps);
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One CTA per probe (grid-stride).  The CTA first derives, in float64, its
// constants (float32 copies of the distances and the focal power, the scan
// rotation) and its probe's scan position and combined Scanner + Descanner
// shift (grid.py:155-182 ScanGrid map, the descan rows), so no separate
// set-up launch runs; then the chain and its hand-derived adjoint per ray in
// float32 registers; the probe's eight sums leave as float64.
__global__ void __launch_bounds__(kFitThreads) k_stem_fit(const __grid_constant__ FitArgs A) {
  __shared__ float wsum[kFitThreads / 32][8];
  __shared__ float4 s_shift;
  __shared__ float s_par[4];
  __shared__ double s_rot[2];
  // the reduction's counters, zeroed before it runs (stream order)
  if (blockIdx.x == 0 && threadIdx.x <= kFitOut) A.cnt[threadIdx.x] = 0;
  // two float64 chains in two warps, so they run side by side
  if (threadIdx.x == 0) {
    double sr, cr;
    sincospi(A.theta[3] / 180.0, &sr, &cr);  // degrees: an exact argument reduction
    s_rot[0] = cr;
    s_rot[1] = sr;
    if (blockIdx.x == 0) A.rot[0] = make_double2(cr, sr);
  } else if (threadIdx.x == 32) {
    s_par[0] = (float)A.theta[1];
    s_par[1] = (float)(A.theta[2] - A.gap);
    s_par[2] = (float)(1.0 / A.theta[0]);
    s_par[3] = (float)A.gap;
  }
  __syncthreads();
  const float D = s_par[0], Lp = s_par[1], invf = s_par[2], G = s_par[3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p = blockIdx.x; p < A.n_probes; p += gridDim.x) {
    __syncthreads();  // the previous probe's threads have read s_shift
    if (threadIdx.x == 0) {
      const double cr = s_rot[0], sr = s_rot[1], step = A.theta[4];
      const double u = (double)(p / A.cols) - 0.5 * (A.rows - 1), v = (double)(p % A.cols) - 0.5 * (A.cols - 1);
      const double spx = step * (-sr * u + cr * v);
      const double spy = -step * (cr * u + sr * v);
      A.sp[p] = make_double2(spx, spy);
      const double* M = A.theta + 5;
      s_shift = make_float4((float)(M[0] * spx + M[1] * spy), (float)(M[4] * spx + M[5] * spy),
                            (float)(M[8] * spx + M[9] * spy), (float)(M[12] * spx + M[13] * spy));
    }
    __syncthreads();
    const float4 sh = s_shift;
    // per-thread sums: loss, dL/dLp, dL/df, dL/dD, Gx, Gy, Gdx, Gdy
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = threadIdx.x; i < A.n; i += blockDim.x) {
      const float x0 = A.x[i], y0 = A.y[i], dx0 = A.dx[i], dy0 = A.dy[i];
      const float x2 = fmaf(dx0, D, x0) + sh.x, y2 = fmaf(dy0, D, y0) + sh.y;
      const float dx2 = dx0 + sh.z, dy2 = dy0 + sh.w;
      const float x3 = fmaf(dx2, G, x2), y3 = fmaf(dy2, G, y2);
      const float dx4 = fmaf(-x3, invf, dx2), dy4 = fmaf(-y3, invf, dy2);
      const float xd = fmaf(dx4, Lp, x3), yd = fmaf(dy4, Lp, y3);
      const size_t o = (size_t)p * A.n + i;
      if (A.forward_only) {
        if (A.ox) A.ox[o] = xd;
        if (A.oy) A.oy[o] = yd;
        continue;
      }
      const float rx = xd - A.tx[o], ry = yd - A.ty[o];
      s[0] += rx * rx + ry * ry;
      const float lxd = 2.f * rx, lyd = 2.f * ry;
      s[1] += lxd * dx4 + lyd * dy4;                    // dL/dLp
      const float ldx4 = lxd * Lp, ldy4 = lyd * Lp;
      s[2] += (ldx4 * x3 + ldy4 * y3) * (invf * invf);  // dL/df
      const float lx3 = lxd - ldx4 * invf, ly3 = lyd - ldy4 * invf;
      const float ldx2 = fmaf(lx3, G, ldx4), ldy2 = fmaf(ly3, G, ldy4);
      s[3] += lx3 * dx0 + ly3 * dy0;                    // dL/dD (lambda_x2 = lambda_x3)
      s[4] += lx3;
      s[5] += ly3;
      s[6] += ldx2;
      s[7] += ldy2;
    }
    if (A.forward_only) continue;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float v = warp_sumf(s[k]);
      if (lane == 0) wsum[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += (double)wsum[w][threadIdx.x];
      A.psum[(size_t)p * 8 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// out[j] for j = blockIdx.x: loss (j = 0) or dL/dtheta[j-1], from the
// per-probe sums through the scan-geometry chain rule (float64).  Each of
// the kRedChunks blocks of an output (blockIdx.y) reduces one chunk of probes
// with a fixed-order tree; the block that counts an output's last chunk adds
// the chunk partials in chunk order (deterministic).  Spreading the float64
// work over kFitOut x kRedChunks blocks matters on GB300, whose float64 rate
// is ~1/64 of float32.
__global__ void __launch_bounds__(128) k_fit_reduce(const __grid_constant__ FitArgs A, double* __restrict__ out) {
  __shared__ double red[128];
  __shared__ int s_last;
  const int j = blockIdx.x, chunk = blockIdx.y;
  const double cr = A.rot[0].x, sr = A.rot[0].y, step = A.theta[4];
  const double* M = A.theta + 5;
  const double kdeg = 3.141592653589793 / 180.0;
  const int per = (A.n_probes + kRedChunks - 1) / kRedChunks;
  const int p0 = chunk * per, p1 = (p0 + per) < A.n_probes ? (p0 + per) : A.n_probes;
  double acc = 0.0;
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    const double* t = A.psum + (size_t)p * 8;
    double c = 0.0;
    if (j == 0) c = t[0];
    else if (j == 1) c = t[2];
    else if (j == 2) c = t[3];
    else if (j == 3) c = t[1];
    else if (j == 4 || j == 5) {
      const double u = (double)(p / A.cols) - 0.5 * (A.rows - 1), v = (double)(p % A.cols) - 0.5 * (A.cols - 1);
      double gsx = 0.0, gsy = 0.0;
      for (int r = 0; r < 4; ++r) {
        gsx += t[4 + r] * M[4 * r + 0];
        gsy += t[4 + r] * M[4 * r + 1];
      }
      if (j == 4) c = gsx * (step * kdeg * (-cr * u - sr * v)) + gsy * (-step * kdeg * (-sr * u + cr * v));
      else c = gsx * (-sr * u + cr * v) + gsy * (-(cr * u + sr * v));
    } else {
      const int e = j - 6, r = e >> 2, col = e & 3;  // dL/dM[r][col]; tilt columns multiply zero tilt
      if (col < 2) c = t[4 + r] * (col == 0 ? A.sp[p].x : A.sp[p].y);
    }
    acc += c;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    A.part[j * kRedChunks + chunk] = red[0];
    __threadfence();
    s_last = atomicAdd(A.cnt + j, 1) == kRedChunks - 1;
  }
  __syncthreads();
  __shared__ int s_adam;
  if (threadIdx.x == 0) {
    s_adam = 0;
    if (s_last) {
      __threadfence();
      double t = 0.0;
      for (int c = 0; c < kRedChunks; ++c) t += __ldcg(A.part + j * kRedChunks + c);
      out[j] = t;
      // the block completing the last output runs the Adam update: every
      // block has finished reading theta by then
      if (A.adam) {
        __threadfence();
        s_adam = atomicAdd(A.cnt + kFitOut, 1) == kFitOut - 1;
      }
    }
  }
  __syncthreads();
  if (s_adam) {
    __threadfence();
    __shared__ double s_c[2];
    __shared__ int64_t s_tt;
    if (threadIdx.x == 0) {
      s_tt = *A.t + 1;
      s_c[0] = 1.0 - powi(A.b1, s_tt);
      s_c[1] = 1.0 - powi(A.b2, s_tt);
    }
    __syncthreads();
    if (threadIdx.x < kFitOut - 1)
      adam_update(threadIdx.x, A.theta_w, __ldcg(out + 1 + threadIdx.x), A.m, A.v, A.lr, A.b1, A.b2,
                  A.eps, s_c[0], s_c[1], A.scale, A.mask);
    if (threadIdx.x == 0) *A.t = s_tt;
  }
}

// Adam on float64 parameters; the step counter lives on the device so the
// update can be replayed inside a CUDA graph.  mask: 1 = parameter is fitted.
__global__ void k_adam(double* __restrict__ theta, const double* __restrict__ grad, double* __restrict__ m,
                       double* __restrict__ v, int64_t* __restrict__ t, int n, double lr, double b1,
                       double b2, double eps, const double* __restrict__ scale,
                       const uint8_t* __restrict__ mask) {
  __shared__ int64_t tt;
  __shared__ double c[2];
  if (threadIdx.x == 0) {
    tt = *t + 1;
    c[0] = 1.0 - powi(b1, tt);
    c[1] = 1.0 - powi(b2, tt);
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (i < n) adam_update(i, theta, grad[i], m, v, lr, b1, b2, eps, c[0], c[1], scale, mask);
  __syncthreads();
  if (threadIdx.x == 0) *t = tt;
}

static int fit_grid(int n_probes) {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
    if (cached <= 0) cached = 148;
  }
  // one probe per CTA up to eight CTAs per SM (all resident in one wave)
  int g = cached * 8;
  return g < n_probes ? g : (n_probes > 0 ? n_probes : 1);
}

// workspace: reserved [n_probes] float4 | sp [n_probes] double2 | psum [n_probes][8] |
// rot (256 B) | part [kFitOut][kRedChunks] | cnt [kFitOut + 1] (256 B)
static size_t fit_ws(int32_t n_probes) {
  return (size_t)n_probes * (16 + 16 + 64) + 256 + kFitOut * kRedChunks * sizeof(double) + 256;
}

}  // namespace tg

using namespace tg;

extern "C" size_t tg_stem_fit_workspace(int32_t n_probes) {
  if (n_probes <= 0) return 0;
  return fit_ws(n_probes);
}

static int fit_args(const tg_stem_fit* c, const double* theta, void* ws, size_t ws_bytes, FitArgs* A) {
  if (!c || !theta) return TG_ERR_INVALID;
  if (c->n_rays < 0 || c->rows <= 0 || c->cols <= 0) return TG_ERR_INVALID;
  if (c->n_rays > 0 && (!c->x || !c->y || !c->dx || !c->dy)) return TG_ERR_INVALID;
  std::memset(A, 0, sizeof(*A));
  A->n = c->n_rays;
  A->rows = c->rows;
  A->cols = c->cols;
  A->n_probes = c->rows * c->cols;
  if (!ws || ws_bytes < fit_ws(A->n_probes)) return TG_ERR_WORKSPACE;
  if (((uintptr_t)ws & 15) != 0) return TG_ERR_ALIGN;
  A->x = c->x; A->y = c->y; A->dx = c->dx; A->dy = c->dy;
  A->tx = c->target_x;
  A->ty = c->target_y;
  A->theta = theta;
  A->gap = c->lens_gap;
  char* w = reinterpret_cast<char*>(ws);
  A->sp = reinterpret_cast<double2*>(w + (size_t)A->n_probes * 16);
  A->psum = reinterpret_cast<double*>(w + (size_t)A->n_probes * 32);
  A->rot = reinterpret_cast<double2*>(w + (size_t)A->n_probes * 96 + 16);
  A->part = reinterpret_cast<double*>(w + (size_t)A->n_probes * 96 + 256);
  A->cnt = reinterpret_cast<int32_t*>(w + (size_t)A->n_probes * 96 + 256 + kFitOut * kRedChunks * sizeof(double));
  return TG_OK;
}

extern "C" int tg_stem_fit_forward(const tg_stem_fit* cfg, const double* theta, float* det_x,
                                   float* det_y, void* workspace, size_t ws_bytes, void* stream) {
  FitArgs A;
  int st = fit_args(cfg, theta, workspace, ws_bytes, &A);
  if (st != TG_OK) return st;
  if (!det_x || !det_y) return TG_ERR_INVALID;
  A.forward_only = 1;
  A.ox = det_x;
  A.oy = det_y;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_stem_fit<<<fit_grid(A.n_probes), kFitThreads, 0, s>>>(A);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_stem_fit_loss_grad(const tg_stem_fit* cfg, const double* theta, double* out,
                                     void* workspace, size_t ws_bytes, void* stream) {
  FitArgs A;
  int st = fit_args(cfg, theta, workspace, ws_bytes, &A);
  if (st != TG_OK) return st;
  if (!out || (A.n > 0 && (!A.tx || !A.ty))) return TG_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_stem_fit<<<fit_grid(A.n_probes), kFitThreads, 0, s>>>(A);
  k_fit_reduce<<<dim3(kFitOut, kRedChunks), 128, 0, s>>>(A, out);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_stem_fit_step(const tg_stem_fit* cfg, double* theta, double* out, double* m,
                                double* v, int64_t* t, double lr, double beta1, double beta2,
                                double eps, const double* scale, const uint8_t* mask,
                                void* workspace, size_t ws_bytes, void* stream) {
  FitArgs A;
  int st = fit_args(cfg, theta, workspace, ws_bytes, &A);
  if (st != TG_OK) return st;
  if (!out || !m || !v || !t || (A.n > 0 && (!A.tx || !A.ty))) return TG_ERR_INVALID;
  A.adam = 1;
  A.theta_w = theta;
  A.m = m;
  A.v = v;
  A.t = t;
  A.lr = lr;
  A.b1 = beta1;
  A.b2 = beta2;
  A.eps = eps;
  A.scale = scale;
  A.mask = mask;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_stem_fit<<<fit_grid(A.n_probes), kFitThreads, 0, s>>>(A);
  k_fit_reduce<<<dim3(kFitOut, kRedChunks), 128, 0, s>>>(A, out);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}

extern "C" int tg_adam_step(double* theta, const double* grad, double* m, double* v, int64_t* t,
                            int32_t n, double lr, double beta1, double beta2, double eps,
                            const double* scale, const uint8_t* mask, void* stream) {
  if (!theta || !grad || !m || !v || !t || n <= 0 || n > 1024) return TG_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_adam<<<1, ((n + 31) / 32) * 32, 0, s>>>(theta, grad, m, v, t, n, lr, beta1, beta2, eps, scale, mask);
  return cudaGetLastError() == cudaSuccess ? TG_OK : TG_ERR_CUDA;
}
