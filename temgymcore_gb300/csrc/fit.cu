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
// k_stem_fit: one CTA per probe at a time; each thread runs the chain and its
// hand-derived adjoint for its rays in registers, the CTA reduces the probe's
// sums, and one thread applies the chain rule through the scan geometry in
// float64.  Per-CTA partials are reduced in fixed order (deterministic).
#include <cstring>

#include "tg_common.cuh"

TG_DEFINE_ERROR_WORD(fit)

namespace tg {

constexpr int kFitThreads = 256;
constexpr int kFitOut = 22;  // loss + 21 gradients

struct FitArgs {
  int32_t n, rows, cols, n_probes;
  const float *x, *y, *dx, *dy;
  const float *tx, *ty;  // [n_probes][n]
  float *ox, *oy;        // forward mode outputs [n_probes][n] (may be NULL)
  const double* theta;
  double gap;
  double* partial;  // [gridDim.x][kFitOut]
  int32_t forward_only;
};

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kFitThreads)
k_stem_fit(const __grid_constant__ FitArgs A) {
  __shared__ double th[21];
  __shared__ double acc[kFitOut];
  __shared__ float wsum[kFitThreads / 32][8];
  __shared__ float4 shift;  // per-probe combined scanner+descanner shift
  __shared__ double sp[2];
  __shared__ double trig[2];   // cos, sin of the scan rotation
  __shared__ float fpar[4];    // D, Lp, 1/f (float32 copies)
  // float64 set-up by one thread: GB300's float64 rate is ~1/60 of float32,
  // so no per-thread float64 transcendental or division is issued.
  if (threadIdx.x < 21) th[threadIdx.x] = A.theta[threadIdx.x];
  if (threadIdx.x < kFitOut) acc[threadIdx.x] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr_, cr_;
    sincos(th[3] * (3.141592653589793 / 180.0), &sr_, &cr_);
    trig[0] = cr_;
    trig[1] = sr_;
    fpar[0] = (float)th[1];
    fpar[1] = (float)(th[2] - A.gap);
    fpar[2] = (float)(1.0 / th[0]);
  }
  __syncthreads();
  const float D = fpar[0], Lp = fpar[1], invf = fpar[2];
  const float G = (float)A.gap;
  const double PI = 3.141592653589793;
  const double cr = trig[0], sr = trig[1];
  const double step = th[4];
  const double r0 = 0.5 * (A.rows - 1), c0 = 0.5 * (A.cols - 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p = blockIdx.x; p < A.n_probes; p += gridDim.x) {
    if (threadIdx.x == 0) {
      const double u = (double)(p / A.cols) - r0, v = (double)(p % A.cols) - c0;
      const double spx = step * (-sr * u + cr * v);
      const double spy = -step * (cr * u + sr * v);
      sp[0] = spx;
      sp[1] = spy;
      const double* M = th + 5;
      shift = make_float4((float)(M[0] * spx + M[1] * spy), (float)(M[4] * spx + M[5] * spy),
                          (float)(M[8] * spx + M[9] * spy), (float)(M[12] * spx + M[13] * spy));
    }
    __syncthreads();
    const float4 sh = shift;
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
      s[1] += lxd * dx4 + lyd * dy4;              // dL/dLp
      const float ldx4 = lxd * Lp, ldy4 = lyd * Lp;
      s[2] += (ldx4 * x3 + ldy4 * y3) * (invf * invf);  // dL/df
      const float lx3 = lxd - ldx4 * invf, ly3 = lyd - ldy4 * invf;
      const float ldx2 = fmaf(lx3, G, ldx4), ldy2 = fmaf(ly3, G, ldy4);
      s[3] += lx3 * dx0 + ly3 * dy0;              // dL/dD (lambda_x2 = lambda_x3)
      s[4] += lx3;
      s[5] += ly3;
      s[6] += ldx2;
      s[7] += ldy2;
    }
    if (!A.forward_only) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        float v = warp_sumf(s[k]);
        if (lane == 0) wsum[warp][k] = v;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
          for (int k = 0; k < 8; ++k) t[k] += (double)wsum[w][k];
        const double* M = th + 5;
        const double spx = sp[0], spy = sp[1];
        const double u = (double)(p / A.cols) - r0, v = (double)(p % A.cols) - c0;
        acc[0] += t[0];
        acc[1] += t[2];                 // f
        acc[2] += t[3];                 // defocus
        acc[3] += t[1];                 // camera length (Lp = CL - gap)
        const double gr[4] = {t[4], t[5], t[6], t[7]};
        double gsx = 0.0, gsy = 0.0;
        for (int r = 0; r < 4; ++r) {
          gsx += gr[r] * M[4 * r + 0];
          gsy += gr[r] * M[4 * r + 1];
          acc[6 + 4 * r + 0] += gr[r] * spx;  // dL/dM[r][0]
          acc[6 + 4 * r + 1] += gr[r] * spy;  // dL/dM[r][1]
          // tilt columns multiply a zero scan tilt: zero gradient
        }
        const double k = PI / 180.0;
        acc[4] += gsx * (step * k * (-cr * u - sr * v)) + gsy * (-step * k * (-sr * u + cr * v));  // rot
        acc[5] += gsx * (-sr * u + cr * v) + gsy * (-(cr * u + sr * v));                         // step
      }
    }
    __syncthreads();
  }
  if (!A.forward_only && threadIdx.x < kFitOut)
    A.partial[(size_t)blockIdx.x * kFitOut + threadIdx.x] = acc[threadIdx.x];
}

// out[0] = loss, out[1..21] = dL/dtheta (sum of block partials in block order)
__global__ void k_fit_reduce(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  const int i = threadIdx.x;
  if (i >= kFitOut) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * kFitOut + i];
  out[i] = s;
}

// Adam on float64 parameters; the step counter lives on the device so the
// update can be replayed inside a CUDA graph.  mask: 1 = parameter is fitted.
__global__ void k_adam(double* __restrict__ theta, const double* __restrict__ grad, double* __restrict__ m,
                       double* __restrict__ v, int64_t* __restrict__ t, int n, double lr, double b1,
                       double b2, double eps, const double* __restrict__ scale,
                       const uint8_t* __restrict__ mask) {
  __shared__ int64_t tt;
  if (threadIdx.x == 0) tt = *t + 1;
  __syncthreads();
  const int i = threadIdx.x;
  if (i < n && (!mask || mask[i])) {
    // gradients w.r.t. parameters normalised by their scale (Adam in relative units)
    const double sc = scale ? scale[i] : 1.0;
    const double g = grad[i] * sc;
    m[i] = b1 * m[i] + (1.0 - b1) * g;
    v[i] = b2 * v[i] + (1.0 - b2) * g * g;
    const double mh = m[i] / (1.0 - pow(b1, (double)tt));
    const double vh = v[i] / (1.0 - pow(b2, (double)tt));
    theta[i] -= sc * lr * mh / (sqrt(vh) + eps);
  }
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
  int g = cached * 4;
  return g < n_probes ? g : (n_probes > 0 ? n_probes : 1);
}

}  // namespace tg

using namespace tg;

extern "C" size_t tg_stem_fit_workspace(int32_t n_probes) {
  if (n_probes <= 0) return 0;
  return (size_t)fit_grid(n_probes) * kFitOut * sizeof(double);
}

static int fit_args(const tg_stem_fit* c, const double* theta, FitArgs* A) {
  if (!c || !theta) return TG_ERR_INVALID;
  if (c->n_rays < 0 || c->rows <= 0 || c->cols <= 0) return TG_ERR_INVALID;
  if (c->n_rays > 0 && (!c->x || !c->y || !c->dx || !c->dy)) return TG_ERR_INVALID;
  std::memset(A, 0, sizeof(*A));
  A->n = c->n_rays;
  A->rows = c->rows;
  A->cols = c->cols;
  A->n_probes = c->rows * c->cols;
  A->x = c->x; A->y = c->y; A->dx = c->dx; A->dy = c->dy;
  A->tx = c->target_x;
  A->ty = c->target_y;
  A->theta = theta;
  A->gap = c->lens_gap;
  return TG_OK;
}

extern "C" int tg_stem_fit_forward(const tg_stem_fit* cfg, const double* theta, float* det_x,
                                   float* det_y, void* stream) {
  FitArgs A;
  int st = fit_args(cfg, theta, &A);
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
  int st = fit_args(cfg, theta, &A);
  if (st != TG_OK) return st;
  if (!out || (A.n > 0 && (!A.tx || !A.ty))) return TG_ERR_INVALID;
  const int grid = fit_grid(A.n_probes);
  if (!workspace || ws_bytes < (size_t)grid * kFitOut * sizeof(double)) return TG_ERR_WORKSPACE;
  A.partial = reinterpret_cast<double*>(workspace);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  k_stem_fit<<<grid, kFitThreads, 0, s>>>(A);
  k_fit_reduce<<<1, 32, 0, s>>>(A.partial, grid, out);
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
