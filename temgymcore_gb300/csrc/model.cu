// model.cpp - host side of the C ABI: model compilation, float64 ABCD
// composition, status strings and the device error word.
//
// compile_program() turns the caller's component list into the Program the
// kernels execute (see tg_common.cuh).  It mirrors run.py:75-82: before every
// component a free-space step of distance (component.z - ray.z), applied even
// when that distance is 0; z then advances by that distance.
#include <cmath>
#include <cstring>

#include "tg_common.cuh"

namespace tg {

static inline double sq(double v) { return v * v; }

// Per-probe shift rows for the Scanner / Descanner: Delta_r = a*spx + b*spy + c.
static void probe_rows(const tg_component& c, double rows[12]) {
  const double* p = c.p;
  double stx = p[2], sty = p[3];
  if (c.kind == TG_SCANNER) {
    double r[12] = {1, 0, 0, 0, 1, 0, 0, 0, stx, 0, 0, sty};
    std::memcpy(rows, r, sizeof(r));
    return;
  }
  const double* M = p + 4;   // 4x4 row-major
  const double* off = p + 20;
  double st[2] = {stx, sty};
  for (int r = 0; r < 4; ++r) {
    double a = M[4 * r + 0], b = M[4 * r + 1];
    double cst = M[4 * r + 2] * st[0] + M[4 * r + 3] * st[1] + off[r];
    if (r == 0) a -= 1.0;
    if (r == 1) b -= 1.0;
    if (r == 2) cst -= stx;
    if (r == 3) cst -= sty;
    rows[3 * r + 0] = a;
    rows[3 * r + 1] = b;
    rows[3 * r + 2] = cst;
  }
}

// Descanner offsets for a fixed scan position, in the reference's operation
// order (components.py:346-372): ((spx*m0 + spy*m1) + off) - sp.
static void descan_delta(const tg_component& c, double d[4]) {
  const double* p = c.p;
  double spx = p[0], spy = p[1], stx = p[2], sty = p[3];
  const double* M = p + 4;
  const double* off = p + 20;
  double sub[4] = {spx, spy, stx, sty};
  for (int r = 0; r < 4; ++r) {
    double v = ((spx * M[4 * r] + spy * M[4 * r + 1]) + off[r]) - sub[r];
    if (M[4 * r + 2] != 0.0 || M[4 * r + 3] != 0.0)
      v += stx * M[4 * r + 2] + sty * M[4 * r + 3];
    d[r] = v;
  }
}

int component_affine_f64(const tg_component& c, double cm[25]) {
  std::memset(cm, 0, 25 * sizeof(double));
  for (int i = 0; i < 5; ++i) cm[6 * i] = 1.0;
  const double* p = c.p;
  switch (c.kind) {
    case TG_PLANE:
    case TG_APERTURE:
    case TG_BIPRISM:  // its offset def_x * sign(x) depends on the ray: callers add it
      return TG_OK;
    case TG_LENS:
    case TG_THICKLENS:
      if (!(p[0] != 0.0)) return TG_ERR_INVALID;
      cm[10] = -1.0 / p[0];  // [2,0]
      cm[16] = -1.0 / p[0];  // [3,1]
      return TG_OK;
    case TG_SCANNER:
    case TG_DESCANNER: {
      if (c.flags & TG_FLAG_PER_PROBE) return TG_ERR_UNSUPPORTED;
      double d[4];
      if (c.kind == TG_SCANNER) {
        d[0] = p[0]; d[1] = p[1]; d[2] = p[2]; d[3] = p[3];
      } else {
        descan_delta(c, d);
      }
      for (int r = 0; r < 4; ++r) cm[5 * r + 4] = d[r];
      return TG_OK;
    }
    case TG_DEFLECTOR:
      cm[14] = p[0];  // [2,4]
      cm[19] = p[1];  // [3,4]
      return TG_OK;
    case TG_ROTATOR: {
      const double a = p[0] * (M_PI / 180.0), ca = std::cos(a), sa = std::sin(a);
      cm[0] = ca; cm[1] = -sa; cm[5] = sa; cm[6] = ca;
      cm[12] = ca; cm[13] = -sa; cm[17] = sa; cm[18] = ca;
      return TG_OK;
    }
    default:
      return TG_ERR_UNSUPPORTED;
  }
}

int compile_program(const tg_model* model, bool per_ray_z, double z_scalar,
                    Program* prog) {
  if (!model || !prog || model->n_components < 0 ||
      (model->n_components > 0 && !model->components))
    return TG_ERR_INVALID;
  if (model->n_components > TG_MAX_COMPONENTS) return TG_ERR_TOO_LARGE;
  if (model->propagator != TG_PROP_PARAXIAL && model->propagator != TG_PROP_DIRCOS)
    return TG_ERR_INVALID;
  std::memset(prog, 0, sizeof(Program));
  prog->dircos = model->propagator == TG_PROP_DIRCOS;
  const int nc = model->n_components;
  prog->n_steps = 2 * nc;
  double z = z_scalar;
  double pl = 0.0;
  for (int i = 0; i < nc; ++i) {
    const tg_component& c = model->components[i];
    Op& fo = prog->op[2 * i];
    Op& co = prog->op[2 * i + 1];
    prog->comp_kind[2 * i] = -1;
    prog->comp_kind[2 * i + 1] = c.kind;
    fo.aux = prog->dircos;  // 1: direction-cosine propagation
    if (i == 0 && per_ray_z) {
      fo.kind = OP_FREE_VARZ;
      prog->zc_first = c.z;
      z = c.z;
    } else {
      double d = c.z - z;
      fo.kind = OP_FREE;
      fo.c[0] = (float)d;
      prog->dstep[2 * i] = d;
      pl += d;
      z = z + d;
    }
    const double* p = c.p;
    bool probe = (c.flags & TG_FLAG_PER_PROBE) != 0;
    if (probe && c.kind != TG_SCANNER && c.kind != TG_DESCANNER) return TG_ERR_UNSUPPORTED;
    switch (c.kind) {
      case TG_PLANE:
        co.kind = OP_NOP;
        break;
      case TG_LENS:
      case TG_THICKLENS: {
        double f = p[0];
        if (!(f != 0.0)) return TG_ERR_INVALID;
        co.kind = OP_LENS;
        co.c[0] = (float)(1.0 / f);
        co.c[1] = (float)(1.0 / (2.0 * f));
        if (c.kind == TG_THICKLENS) z = z - (c.z - p[1]);
      } break;
      case TG_SCANNER:
      case TG_DESCANNER:
        if (probe) {
          if (prog->n_probe_ops >= kMaxProbeOps) return TG_ERR_TOO_LARGE;
          co.kind = OP_PROBE_SHIFT;
          co.aux = prog->n_probe_ops;
          probe_rows(c, prog->pcoef[prog->n_probe_ops]);
          prog->n_probe_ops++;
        } else {
          co.kind = OP_SHIFT;
          double d[4];
          if (c.kind == TG_SCANNER) {
            d[0] = p[0]; d[1] = p[1]; d[2] = p[2]; d[3] = p[3];
          } else {
            descan_delta(c, d);
          }
          for (int k = 0; k < 4; ++k) co.c[k] = (float)d[k];
        }
        break;
      case TG_DEFLECTOR:
        co.kind = OP_DEFLECT;
        co.c[0] = (float)p[0];
        co.c[1] = (float)p[1];
        break;
      case TG_BIPRISM:
        if (prog->n_biprism >= 32) return TG_ERR_TOO_LARGE;
        co.kind = OP_BIPRISM;
        co.aux = prog->n_biprism++;
        co.c[0] = (float)p[0];
        break;
      case TG_ROTATOR: {
        double a = p[0] * (M_PI / 180.0);
        co.kind = OP_ROTATE;
        co.c[0] = (float)std::cos(a);
        co.c[1] = (float)std::sin(a);
      } break;
      case TG_APERTURE:
        co.kind = OP_APERTURE;
        co.c[0] = (float)sq(p[0]);
        co.c[1] = (float)p[1];
        co.c[2] = (float)p[2];
        prog->has_aperture = 1;
        break;
      case TG_ABERLENS: {
        double f = p[0];
        if (!(f != 0.0)) return TG_ERR_INVALID;
        if (prog->n_aber >= kMaxAber) return TG_ERR_TOO_LARGE;
        co.kind = OP_ABER;
        co.aux = prog->n_aber;
        co.c[0] = (float)(1.0 / f);
        co.c[1] = (float)(1.0 / (2.0 * f));
        double w[kAberW], gx[kAberG], gy[kAberG];
        aber_monomials(p + 1, w);
        aber_gradient(w, gx, gy);
        float* a = prog->aber[prog->n_aber++];
        for (int k = 0; k < kAberW; ++k) a[k] = (float)w[k];
        for (int k = 0; k < kAberG; ++k) a[kAberW + k] = (float)gx[k];
        for (int k = 0; k < kAberG; ++k) a[kAberW + kAberG + k] = (float)gy[k];
      } break;
      default:
        return TG_ERR_UNSUPPORTED;
    }
  }
  prog->pl_const = pl;
  prog->z_out = z;
  return TG_OK;
}

}  // namespace tg

using namespace tg;

// ------------------------------------------------------------ float64 ABCD
static void mat5_mul(const double a[25], const double b[25], double out[25]) {
  double t[25];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) s += a[5 * i + k] * b[5 * k + j];
      t[5 * i + j] = s;
    }
  std::memcpy(out, t, sizeof(t));
}

static void eye5(double m[25]) {
  std::memset(m, 0, 25 * sizeof(double));
  for (int i = 0; i < 5; ++i) m[6 * i] = 1.0;
}

extern "C" int tg_abcd_compose(const tg_model* model, const double central[5],
                               double out[25], double* steps) {
  if (!model || !central || !out) return TG_ERR_INVALID;
  if (model->propagator != TG_PROP_PARAXIAL && model->propagator != TG_PROP_DIRCOS)
    return TG_ERR_INVALID;
  if (model->n_components < 0 || model->n_components > TG_MAX_COMPONENTS)
    return TG_ERR_INVALID;
  if (model->n_components > 0 && !model->components) return TG_ERR_INVALID;
  // central ray in float64 (x, y, dx, dy, z)
  double x = central[0], y = central[1], dx = central[2], dy = central[3], z = central[4];
  double total[25];
  eye5(total);
  for (int i = 0; i < model->n_components; ++i) {
    const tg_component& c = model->components[i];
    const double* p = c.p;
    double d = c.z - z;
    double fm[25];
    eye5(fm);
    if (model->propagator == TG_PROP_DIRCOS) {
      // x' = x + d dx / n2, n2 = 1 + dx^2 + dy^2 (propagator.py:100-110)
      const double n2 = 1.0 + dx * dx + dy * dy, inv = 1.0 / n2, inv2 = inv * inv;
      fm[2] = d * (inv - 2.0 * dx * dx * inv2);  // [0,2]
      fm[3] = -2.0 * d * dx * dy * inv2;         // [0,3]
      fm[5 + 2] = -2.0 * d * dx * dy * inv2;     // [1,2]
      fm[5 + 3] = d * (inv - 2.0 * dy * dy * inv2);  // [1,3]
      mat5_mul(fm, total, total);
      if (steps) std::memcpy(steps + 50 * i, fm, sizeof(fm));
      x += dx * inv * d;
      y += dy * inv * d;
    } else {
      fm[2] = d;       // [0,2]
      fm[5 + 3] = d;   // [1,3]
      mat5_mul(fm, total, total);
      if (steps) std::memcpy(steps + 50 * i, fm, sizeof(fm));
      x += dx * d;
      y += dy * d;
    }
    z += d;
    double cm[25];
    eye5(cm);
    switch (c.kind) {
      case TG_PLANE:
      case TG_APERTURE:
        break;
      case TG_LENS:
      case TG_THICKLENS: {
        double f = p[0];
        cm[10] = -1.0 / f;      // [2,0]
        cm[15 + 1] = -1.0 / f;  // [3,1]
        dx = -x / f + dx;
        dy = -y / f + dy;
        if (c.kind == TG_THICKLENS) z = z - (c.z - p[1]);
      } break;
      case TG_SCANNER:
      case TG_DESCANNER: {
        if (c.flags & TG_FLAG_PER_PROBE) return TG_ERR_UNSUPPORTED;
        double dd[4];
        if (c.kind == TG_SCANNER) {
          dd[0] = p[0]; dd[1] = p[1]; dd[2] = p[2]; dd[3] = p[3];
        } else {
          descan_delta(c, dd);
        }
        for (int r = 0; r < 4; ++r) cm[5 * r + 4] = dd[r];
        x += dd[0]; y += dd[1]; dx += dd[2]; dy += dd[3];
      } break;
      case TG_DEFLECTOR:
        cm[14] = p[0];  // [2,4]
        cm[19] = p[1];  // [3,4]
        dx += p[0];
        dy += p[1];
        break;
      case TG_BIPRISM: {
        double s = x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0);
        cm[14] = p[0] * s;
        dx += p[0] * s;
      } break;
      case TG_ABERLENS: {
        // Jacobian of the aberrated lens at the ray: ideal slopes u = d - r/f,
        // d' = u - grad W(u)/f, so d(d')/d(r, d) = (I - H/f) [-I/f, I]
        // with H the Hessian of W at u; no offset column (the aberration
        // does not scale with the ray's _one).
        const double f = p[0];
        if (!(f != 0.0)) return TG_ERR_INVALID;
        const double k1 = 1.0 / f;
        double w[kAberW];
        aber_monomials(p + 1, w);
        const double ux = dx - x * k1, uy = dy - y * k1;
        double W, Wx, Wy, Hxx, Hxy, Hyy;
        aber_eval_f64(w, ux, uy, &W, &Wx, &Wy, &Hxx, &Hxy, &Hyy);
        cm[10] = -k1 + Hxx * k1 * k1;  // [2,0]
        cm[11] = Hxy * k1 * k1;        // [2,1]
        cm[12] = 1.0 - Hxx * k1;       // [2,2]
        cm[13] = -Hxy * k1;            // [2,3]
        cm[15] = Hxy * k1 * k1;        // [3,0]
        cm[16] = -k1 + Hyy * k1 * k1;  // [3,1]
        cm[17] = -Hxy * k1;            // [3,2]
        cm[18] = 1.0 - Hyy * k1;       // [3,3]
        dx = ux - Wx * k1;
        dy = uy - Wy * k1;
      } break;
      case TG_ROTATOR: {
        double a = p[0] * (M_PI / 180.0);
        double ca = std::cos(a), sa = std::sin(a);
        cm[0] = ca; cm[1] = -sa; cm[5] = sa; cm[6] = ca;
        cm[12] = ca; cm[13] = -sa; cm[17] = sa; cm[18] = ca;
        double nx = x * ca - y * sa, ny = x * sa + y * ca;
        double ndx = dx * ca - dy * sa, ndy = dx * sa + dy * ca;
        x = nx; y = ny; dx = ndx; dy = ndy;
      } break;
      default:
        return TG_ERR_UNSUPPORTED;
    }
    mat5_mul(cm, total, total);
    if (steps) std::memcpy(steps + 50 * i + 25, cm, sizeof(cm));
  }
  std::memcpy(out, total, sizeof(total));
  return TG_OK;
}

// ------------------------------------------------------------ library info
extern "C" int tg_aber_monomials(const double* kc, double* w, double* gx, double* gy) {
  if (!kc || !w) return TG_ERR_INVALID;
  aber_monomials(kc, w);
  double g[2][kAberG];
  aber_gradient(w, g[0], g[1]);
  if (gx) std::memcpy(gx, g[0], sizeof(g[0]));
  if (gy) std::memcpy(gy, g[1], sizeof(g[1]));
  return TG_OK;
}

extern "C" const char* tg_version(void) { return "temgym_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* tg_status_string(int s) {
  switch (s) {
    case TG_OK: return "ok";
    case TG_ERR_INVALID: return "invalid argument";
    case TG_ERR_UNSUPPORTED: return "unsupported component or option";
    case TG_ERR_ALIGN: return "pointer alignment requirement violated";
    case TG_ERR_CUDA: return "CUDA runtime error";
    case TG_ERR_TOO_LARGE: return "size beyond the stated maximum";
    case TG_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

extern "C" int tg_internal_err_trace(uint32_t*, int);
extern "C" int tg_internal_err_scan(uint32_t*, int);
extern "C" int tg_internal_err_field(uint32_t*, int);
extern "C" int tg_internal_err_gemm(uint32_t*, int);
extern "C" int tg_internal_err_fit(uint32_t*, int);
extern "C" int tg_internal_err_batch(uint32_t*, int);
extern "C" int tg_internal_err_fadj(uint32_t*, int);

extern "C" int tg_get_error_word(uint32_t* out, int clear);

extern "C" uint32_t tg_get_last_error_word(void) {
  uint32_t v = 0;
  return tg_get_error_word(&v, 1) == TG_OK ? v : 0xffffffffu;
}

extern "C" int tg_get_error_word(uint32_t* out, int clear) {
  if (!out) return TG_ERR_INVALID;
  if (cudaDeviceSynchronize() != cudaSuccess) return TG_ERR_CUDA;
  *out = 0;
  int s = tg_internal_err_trace(out, clear);
  if (s == TG_OK) s = tg_internal_err_scan(out, clear);
  if (s == TG_OK) s = tg_internal_err_field(out, clear);
  if (s == TG_OK) s = tg_internal_err_gemm(out, clear);
  if (s == TG_OK) s = tg_internal_err_fit(out, clear);
  if (s == TG_OK) s = tg_internal_err_batch(out, clear);
  if (s == TG_OK) s = tg_internal_err_fadj(out, clear);
  return s;
}
