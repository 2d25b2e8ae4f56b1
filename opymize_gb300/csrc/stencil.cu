// Finite-difference operators on row-major image grids (generic path):
// gradient / divergence (forward and centered schemes), Laplacian with
// Neumann / curvature / second-order boundaries and their adjoints, and the
// rowwise l^p norms used by diagonal preconditioning.
//
// One thread per output element, grid-stride; neighbour values come through
// L1/L2.  The fused PDHG passes (rof_*.cu) carry their own tiled stencils.
#include "common.cuh"

namespace opyx {

struct GridP {
  int D, C;
  int64_t N;
  int64_t n[OPYX_MAX_DIMS];
  int64_t s[OPYX_MAX_DIMS];
  double invh[OPYX_MAX_DIMS];
};

static int make_grid(const opyx_grid* g, GridP* p) {
  if (!g || g->ndim < 1 || g->ndim > OPYX_MAX_DIMS || g->nchannels < 1) return OPYX_ERR_ARG;
  p->D = g->ndim;
  p->C = g->nchannels;
  int64_t N = 1;
  for (int t = 0; t < p->D; ++t) {
    if (g->dims[t] < 1 || !(g->h[t] > 0)) return OPYX_ERR_ARG;
    p->n[t] = g->dims[t];
    p->invh[t] = 1.0 / g->h[t];
    N *= g->dims[t];
  }
  int64_t s = 1;
  for (int t = p->D - 1; t >= 0; --t) {
    p->s[t] = s;
    s *= p->n[t];
  }
  p->N = N;
  return OPYX_OK;
}

OPYX_D void coords_of(const GridP& g, int64_t i, int64_t* c) {
  for (int t = 0; t < g.D; ++t) c[t] = (i / g.s[t]) % g.n[t];
}

OPYX_D double wk(const double* w, int k) { return w ? __ldg(w + k) : 1.0; }

// Pixel offset of the a-th corner of the averaging cell of axis t: bit b of
// `a` selects +1 along the b-th axis other than t (diff.py:23-42).
OPYX_D int64_t avg_offset(const GridP& g, int t, int a) {
  int64_t off = 0;
  int b = 0;
  for (int u = 0; u < g.D; ++u) {
    if (u == t) continue;
    if ((a >> b) & 1) off += g.s[u];
    ++b;
  }
  return off;
}

// ---- gradient: y[(i*D+t)*C+k] -------------------------------------------
template <typename T>
__global__ void k_gradient(GridP g, int centered, const double* __restrict__ w,
                           const T* __restrict__ x, T* __restrict__ y, int add) {
  const int64_t total = g.N * g.D * g.C;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(o % g.C);
    const int t = (int)((o / g.C) % g.D);
    const int64_t i = o / ((int64_t)g.C * g.D);
    int64_t c[OPYX_MAX_DIMS];
    coords_of(g, i, c);
    T val = T(0);
    if (!centered || g.D == 1) {
      if (c[t] < g.n[t] - 1)
        val = (T)(wk(w, k) * g.invh[t]) * (x[(i + g.s[t]) * g.C + k] - x[i * g.C + k]);
    } else {
      bool inner = true;
      for (int u = 0; u < g.D; ++u) inner &= (c[u] < g.n[u] - 1);
      if (inner) {
        const int navg = 1 << (g.D - 1);
        T acc = T(0);
        for (int a = 0; a < navg; ++a) {
          const int64_t b = i + avg_offset(g, t, a);
          acc += x[(b + g.s[t]) * g.C + k] - x[b * g.C + k];
        }
        val = (T)(wk(w, k) * g.invh[t] / navg) * acc;
      }
    }
    y[o] = add ? y[o] + val : val;
  }
}

// ---- divergence (gradient transpose): x[i*C+k] ---------------------------
template <typename T>
__global__ void k_divergence(GridP g, int centered, const double* __restrict__ w,
                             const T* __restrict__ y, T* __restrict__ x, int add) {
  const int64_t total = g.N * g.C;
  const int64_t dc = (int64_t)g.D * g.C;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(o % g.C);
    const int64_t i = o / g.C;
    int64_t c[OPYX_MAX_DIMS];
    coords_of(g, i, c);
    T acc = T(0);
    if (!centered || g.D == 1) {
      for (int t = 0; t < g.D; ++t) {
        const T ih = (T)g.invh[t];
        if (c[t] < g.n[t] - 1) acc -= y[i * dc + t * g.C + k] * ih;
        if (c[t] > 0) acc += y[(i - g.s[t]) * dc + t * g.C + k] * ih;
      }
    } else {
      const int navg = 1 << (g.D - 1);
      for (int t = 0; t < g.D; ++t) {
        for (int a = 0; a < navg; ++a) {
          // the cell corner i - offset must be an inner gradient pixel in
          // every axis other than t (diff.cu:23-35)
          bool ok = true;
          int b = 0;
          for (int u = 0; u < g.D; ++u) {
            if (u == t) continue;
            const int64_t cu = c[u] - ((a >> b) & 1);
            ok &= (cu >= 0) && (cu != g.n[u] - 1);
            ++b;
          }
          if (!ok) continue;
          const int64_t base = i - avg_offset(g, t, a);
          const T ih = (T)g.invh[t];
          if (c[t] < g.n[t] - 1) acc -= y[base * dc + t * g.C + k] * ih;
          if (c[t] > 0) acc += y[(base - g.s[t]) * dc + t * g.C + k] * ih;
        }
      }
      acc /= (T)navg;
    }
    const T val = (T)wk(w, k) * acc;
    x[o] = add ? x[o] + val : val;
  }
}

OPYX_D double finish_lp(double s, double p) { return p == 1.0 ? s : pow(s, 1.0 / p); }

template <typename T>
__global__ void k_gradient_rowlp(GridP g, int centered, const double* __restrict__ w,
                                 int transpose, double p, T* __restrict__ y, int add) {
  const int64_t total = transpose ? g.N * g.C : g.N * g.D * g.C;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(o % g.C);
    const bool cen = centered && g.D > 1;
    const int navg = cen ? (1 << (g.D - 1)) : 1;
    double s = 0.0;
    int64_t c[OPYX_MAX_DIMS];
    if (!transpose) {
      const int t = (int)((o / g.C) % g.D);
      const int64_t i = o / ((int64_t)g.C * g.D);
      coords_of(g, i, c);
      bool valid = true;
      if (cen) { for (int u = 0; u < g.D; ++u) valid &= (c[u] < g.n[u] - 1); }
      else valid = c[t] < g.n[t] - 1;
      if (valid) s = 2.0 * navg * pow(fabs(wk(w, k) * g.invh[t] / navg), p);
    } else {
      const int64_t i = o / g.C;
      coords_of(g, i, c);
      for (int t = 0; t < g.D; ++t) {
        const double e = pow(fabs(wk(w, k) * g.invh[t] / navg), p);
        const int nt = (c[t] < g.n[t] - 1) + (c[t] > 0);
        if (!cen) { s += nt * e; continue; }
        for (int a = 0; a < navg; ++a) {
          bool ok = true;
          int b = 0;
          for (int u = 0; u < g.D; ++u) {
            if (u == t) continue;
            const int64_t cu = c[u] - ((a >> b) & 1);
            ok &= (cu >= 0) && (cu != g.n[u] - 1);
            ++b;
          }
          if (ok) s += nt * e;
        }
      }
    }
    const double v = finish_lp(s, p);
    y[o] = add ? (T)((double)y[o] + v) : (T)v;
  }
}

// ---- Laplacian --------------------------------------------------------
// Per-axis 1-D second-difference coefficients of row c (length n):
// lo at c-1, up at c+1, dg on the diagonal (sparse.py:28-45, diff.cu:151-240).
OPYX_D void lap1d(int bc, int64_t c, int64_t n, double* lo, double* up, double* dg) {
  if (bc == OPYX_BC_NEUMANN) {
    *lo = c > 0 ? 1.0 : 0.0;
    *up = c < n - 1 ? 1.0 : 0.0;
    *dg = -(*lo) - (*up);
  } else {
    const bool in = c > 0 && c < n - 1;
    *lo = in ? 1.0 : 0.0;
    *up = in ? 1.0 : 0.0;
    *dg = in ? -2.0 : 0.0;
  }
}

OPYX_D bool lap_keep(const GridP& g, int bc, const int64_t* c) {
  if (bc != OPYX_BC_CURVATURE) return true;
  for (int u = 0; u < g.D; ++u)
    if (c[u] == 0 || c[u] == g.n[u] - 1) return false;
  return true;
}

// Row i of L (adjoint = 0) or of L^T (adjoint = 1): diagonal coefficient and
// the coefficients of the neighbours i - s_t (cm[t]) and i + s_t (cp[t]).
OPYX_D void lap_row(const GridP& g, int bc, int adjoint, int64_t* c, double* dg,
                    double* cm, double* cp) {
  const bool keep = lap_keep(g, bc, c);
  double d = 0.0;
  for (int t = 0; t < g.D; ++t) {
    const double ih2 = g.invh[t] * g.invh[t];
    double lo, up, dd;
    lap1d(bc, c[t], g.n[t], &lo, &up, &dd);
    d += dd * ih2;
    if (!adjoint) {
      cm[t] = keep ? lo * ih2 : 0.0;
      cp[t] = keep ? up * ih2 : 0.0;
    } else {
      // L^T[i, i-s_t] = L[i-s_t, i] = up-coefficient of row c_t - 1, etc.
      cm[t] = 0.0;
      cp[t] = 0.0;
      if (c[t] > 0) {
        double l2, u2, d2;
        lap1d(bc, c[t] - 1, g.n[t], &l2, &u2, &d2);
        c[t] -= 1;
        cm[t] = lap_keep(g, bc, c) ? u2 * ih2 : 0.0;
        c[t] += 1;
      }
      if (c[t] < g.n[t] - 1) {
        double l2, u2, d2;
        lap1d(bc, c[t] + 1, g.n[t], &l2, &u2, &d2);
        c[t] += 1;
        cp[t] = lap_keep(g, bc, c) ? l2 * ih2 : 0.0;
        c[t] -= 1;
      }
    }
  }
  *dg = keep ? d : 0.0;
}

template <typename T>
__global__ void k_laplacian(GridP g, int bc, int adjoint, const T* __restrict__ x,
                            T* __restrict__ y, int add) {
  const int64_t total = g.N * g.C;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(o % g.C);
    const int64_t i = o / g.C;
    int64_t c[OPYX_MAX_DIMS];
    double cm[OPYX_MAX_DIMS], cp[OPYX_MAX_DIMS], dg;
    coords_of(g, i, c);
    lap_row(g, bc, adjoint, c, &dg, cm, cp);
    T acc = (T)dg * x[o];
    for (int t = 0; t < g.D; ++t) {
      if (cm[t] != 0.0) acc += (T)cm[t] * x[(i - g.s[t]) * g.C + k];
      if (cp[t] != 0.0) acc += (T)cp[t] * x[(i + g.s[t]) * g.C + k];
    }
    y[o] = add ? y[o] + acc : acc;
  }
}

template <typename T>
__global__ void k_laplacian_rowlp(GridP g, int bc, int adjoint, double p,
                                  T* __restrict__ y, int add) {
  const int64_t total = g.N * g.C;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = o / g.C;
    int64_t c[OPYX_MAX_DIMS];
    double cm[OPYX_MAX_DIMS], cp[OPYX_MAX_DIMS], dg;
    coords_of(g, i, c);
    lap_row(g, bc, adjoint, c, &dg, cm, cp);
    double s = pow(fabs(dg), p);
    for (int t = 0; t < g.D; ++t) s += pow(fabs(cm[t]), p) + pow(fabs(cp[t]), p);
    const double v = finish_lp(s, p);
    y[o] = add ? (T)((double)y[o] + v) : (T)v;
  }
}

}  // namespace opyx

using namespace opyx;

extern "C" {

int opyx_gradient(const opyx_grid* grid, int scheme, const double* w, int dtype,
                  const void* x, void* y, int add, void* stream) {
  GridP g;
  int st = make_grid(grid, &g);
  if (st) return st;
  if (scheme != OPYX_SCHEME_FORWARD && scheme != OPYX_SCHEME_CENTERED) return OPYX_ERR_ARG;
  if (!x || !y) return OPYX_ERR_ARG;
  const int64_t n = g.N * g.D * g.C;
  OPYX_DISPATCH(dtype, T, (k_gradient<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              g, scheme == OPYX_SCHEME_CENTERED, w, (const T*)x, (T*)y, add)));
  return check_launch();
}

int opyx_divergence(const opyx_grid* grid, int scheme, const double* w, int dtype,
                    const void* y, void* x, int add, void* stream) {
  GridP g;
  int st = make_grid(grid, &g);
  if (st) return st;
  if (scheme != OPYX_SCHEME_FORWARD && scheme != OPYX_SCHEME_CENTERED) return OPYX_ERR_ARG;
  if (!x || !y) return OPYX_ERR_ARG;
  const int64_t n = g.N * g.C;
  OPYX_DISPATCH(dtype, T, (k_divergence<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              g, scheme == OPYX_SCHEME_CENTERED, w, (const T*)y, (T*)x, add)));
  return check_launch();
}

int opyx_gradient_rowlp(const opyx_grid* grid, int scheme, const double* w, int transpose,
                        double p, int dtype, void* y, int add, void* stream) {
  GridP g;
  int st = make_grid(grid, &g);
  if (st) return st;
  if (!(p > 0) || !y) return OPYX_ERR_ARG;
  const int64_t n = transpose ? g.N * g.C : g.N * g.D * g.C;
  OPYX_DISPATCH(dtype, T, (k_gradient_rowlp<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              g, scheme == OPYX_SCHEME_CENTERED, w, transpose, p, (T*)y, add)));
  return check_launch();
}

int opyx_laplacian(const opyx_grid* grid, int bc, int adjoint, int dtype, const void* x,
                   void* y, int add, void* stream) {
  GridP g;
  int st = make_grid(grid, &g);
  if (st) return st;
  if (bc < OPYX_BC_NEUMANN || bc > OPYX_BC_SECOND_ORDER || !x || !y) return OPYX_ERR_ARG;
  const int64_t n = g.N * g.C;
  OPYX_DISPATCH(dtype, T, (k_laplacian<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              g, bc, bc == OPYX_BC_NEUMANN ? 0 : adjoint, (const T*)x, (T*)y, add)));
  return check_launch();
}

int opyx_laplacian_rowlp(const opyx_grid* grid, int bc, int adjoint, double p, int dtype,
                         void* y, int add, void* stream) {
  GridP g;
  int st = make_grid(grid, &g);
  if (st) return st;
  if (bc < OPYX_BC_NEUMANN || bc > OPYX_BC_SECOND_ORDER || !(p > 0) || !y) return OPYX_ERR_ARG;
  const int64_t n = g.N * g.C;
  OPYX_DISPATCH(dtype, T, (k_laplacian_rowlp<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
                              g, bc, bc == OPYX_BC_NEUMANN ? 0 : adjoint, p, (T*)y, add)));
  return check_launch();
}

}  // extern "C"
