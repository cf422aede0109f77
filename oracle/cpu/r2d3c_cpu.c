/*
 * r2d3c_cpu.c -- FP64 C/OpenMP restatement of the Rot2D3C time step.
 *
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline of bench.py and a second,
 * independent check of the NumPy oracle.  Nothing in the product links it.
 * Parity status: unpinned (the reference cannot be compiled here; see
 * rot2d3c_oracle.py).
 *
 * It keeps the reference's cost structure on one rank: every poisson call
 * does 4 complex-to-real and 1 real-to-complex 2-D transforms
 * (pseudospec2D_Rot2D3C.f90:169-226), the CFL condition 3 more (:840-899),
 * so one RK4 step costs 35 C2R + 8 R2C, as in Rot2D3C.para.f90:393-611.
 * Threads replace MPI ranks (OpenMP over transform columns/rows).
 *
 * Layouts: spectral C[kx][ky] (n/2+1) x n complex, physical R[y][x] n x n.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} cplx;

typedef struct {
  int n, logn;
  cplx* tw;  /* exp(-2 pi i k/n), k < n/2 */
  int* rev;  /* bit reversal of log2(n) bits */
} fftplan;

static const double PI = 3.1415926535897932384;

static void plan_init(fftplan* p, int n) {
  p->n = n;
  p->logn = 0;
  while ((1 << p->logn) < n) p->logn++;
  p->tw = (cplx*)malloc(sizeof(cplx) * (size_t)(n / 2 > 0 ? n / 2 : 1));
  p->rev = (int*)malloc(sizeof(int) * (size_t)n);
  for (int k = 0; k < n / 2; ++k) {
    p->tw[k].re = cos(2.0 * PI * k / n);
    p->tw[k].im = -sin(2.0 * PI * k / n);
  }
  for (int i = 0; i < n; ++i) {
    int r = 0;
    for (int b = 0; b < p->logn; ++b)
      if (i & (1 << b)) r |= 1 << (p->logn - 1 - b);
    p->rev[i] = r;
  }
}

static void plan_free(fftplan* p) {
  free(p->tw);
  free(p->rev);
}

/* in-place radix-2 DIT, unnormalised; dir = -1 forward, +1 backward */
static void fft1(const fftplan* p, cplx* a, int dir) {
  const int n = p->n;
  for (int i = 0; i < n; ++i) {
    const int j = p->rev[i];
    if (j > i) {
      cplx t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int s = 0; s < n; s += len) {
      for (int k = 0; k < half; ++k) {
        const cplx w = p->tw[k * step];
        const double wi = dir < 0 ? w.im : -w.im;
        cplx* u = &a[s + k];
        cplx* v = &a[s + k + half];
        const double tr = v->re * w.re - v->im * wi;
        const double ti = v->re * wi + v->im * w.re;
        v->re = u->re - tr;
        v->im = u->im - ti;
        u->re += tr;
        u->im += ti;
      }
    }
  }
}

typedef struct {
  int n, nh, threads;
  double kmax, tiny;
  fftplan pl;
  double* ka;  /* ka(i) */
  cplx* t;     /* (n/2+1) x n mixed plane */
} grid;

static void grid_init(grid* g, int n, int threads) {
  g->n = n;
  g->nh = n / 2 + 1;
  g->threads = threads;
  g->kmax = ((double)n / 3.0) * ((double)n / 3.0);
  g->tiny = 0.000001;
  plan_init(&g->pl, n);
  g->ka = (double*)malloc(sizeof(double) * n);
  for (int i = 1; i <= n / 2; ++i) {
    g->ka[i - 1] = (double)(i - 1);
    g->ka[i + n / 2 - 1] = (double)(i - n / 2 - 1);
  }
  g->t = (cplx*)malloc(sizeof(cplx) * (size_t)g->nh * n);
}

static void grid_free(grid* g) {
  plan_free(&g->pl);
  free(g->ka);
  free(g->t);
}

static inline double ka2(const grid* g, int i, int j) { return g->ka[i] * g->ka[i] + g->ka[j] * g->ka[j]; }

/* fftp2d_complex_to_real (fftp2D.f90:214-290): y-IFFT per kx column, then
   x-C2R per row (two rows per complex transform; Im of kx=0, n/2 ignored) */
static void c2r(grid* g, const cplx* in, double* out) {
  const int n = g->n, nh = g->nh;
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (int i = 0; i < nh; ++i) {
    memcpy(&g->t[(size_t)i * n], &in[(size_t)i * n], sizeof(cplx) * n);
    fft1(&g->pl, &g->t[(size_t)i * n], +1);
  }
#pragma omp parallel num_threads(g->threads)
  {
    cplx* z = (cplx*)malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
    for (int pr = 0; pr < n / 2; ++pr) {
      const int y0 = 2 * pr, y1 = y0 + 1;
      for (int k = 0; k < n; ++k) {
        const int kk = k <= n / 2 ? k : n - k;
        const cplx a = g->t[(size_t)kk * n + y0], b = g->t[(size_t)kk * n + y1];
        if (k == 0 || k == n / 2) {
          z[k].re = a.re;
          z[k].im = b.re;
        } else if (k < n / 2) {
          z[k].re = a.re - b.im;
          z[k].im = a.im + b.re;
        } else {
          z[k].re = a.re + b.im;
          z[k].im = b.re - a.im;
        }
      }
      fft1(&g->pl, z, +1);
      for (int x = 0; x < n; ++x) {
        out[(size_t)y0 * n + x] = z[x].re;
        out[(size_t)y1 * n + x] = z[x].im;
      }
    }
    free(z);
  }
}

/* fftp2d_real_to_complex (fftp2D.f90:133-211) */
static void r2c(grid* g, const double* in, cplx* out) {
  const int n = g->n, nh = g->nh;
#pragma omp parallel num_threads(g->threads)
  {
    cplx* z = (cplx*)malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
    for (int pr = 0; pr < n / 2; ++pr) {
      const int y0 = 2 * pr, y1 = y0 + 1;
      for (int x = 0; x < n; ++x) {
        z[x].re = in[(size_t)y0 * n + x];
        z[x].im = in[(size_t)y1 * n + x];
      }
      fft1(&g->pl, z, -1);
      for (int k = 0; k <= n / 2; ++k) {
        const cplx w = z[k], u = z[(n - k) & (n - 1)];
        g->t[(size_t)k * n + y0].re = 0.5 * (w.re + u.re);
        g->t[(size_t)k * n + y0].im = 0.5 * (w.im - u.im);
        g->t[(size_t)k * n + y1].re = 0.5 * (w.im + u.im);
        g->t[(size_t)k * n + y1].im = 0.5 * (u.re - w.re);
      }
    }
    free(z);
  }
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (int i = 0; i < nh; ++i) {
    memcpy(&out[(size_t)i * n], &g->t[(size_t)i * n], sizeof(cplx) * n);
    fft1(&g->pl, &out[(size_t)i * n], -1);
  }
}

/* derivk2 (pseudospec2D_Rot2D3C.f90:6-68) */
static void derivk2(grid* g, const cplx* a, cplx* b, int dir) {
  const int n = g->n;
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (int i = 0; i < g->nh; ++i)
    for (int j = 0; j < n; ++j) {
      const size_t id = (size_t)i * n + j;
      if (ka2(g, i, j) <= g->kmax) {
        const double k = dir == 1 ? g->ka[i] : g->ka[j];
        if (dir == 0) {
          b[id] = a[id];
        } else {
          const cplx x = a[id];
          b[id].re = -k * x.im;
          b[id].im = k * x.re;
        }
      } else {
        b[id].re = 0.0;
        b[id].im = 0.0;
      }
    }
}

/* laplak2 (:71-95) */
static void laplak2(grid* g, const cplx* a, cplx* b) {
  const int n = g->n;
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (int i = 0; i < g->nh; ++i)
    for (int j = 0; j < n; ++j) {
      const size_t id = (size_t)i * n + j;
      const double m = -ka2(g, i, j);
      b[id].re = m * a[id].re;
      b[id].im = m * a[id].im;
    }
}

typedef struct {
  cplx *c1, *c2;
  double *r1, *r2, *r3;
} work;

/* poisson (:169-226) */
static void poisson(grid* g, work* w, const cplx* a, const cplx* b, cplx* c) {
  const size_t nn = (size_t)g->n * g->n;
  const double n4 = (double)g->n * g->n * (double)g->n * g->n;
  derivk2(g, a, w->c1, 1);
  derivk2(g, b, w->c2, 2);
  c2r(g, w->c1, w->r1);
  c2r(g, w->c2, w->r2);
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (size_t i = 0; i < nn; ++i) w->r3[i] = w->r1[i] * w->r2[i];
  derivk2(g, a, w->c1, 2);
  derivk2(g, b, w->c2, 1);
  c2r(g, w->c1, w->r1);
  c2r(g, w->c2, w->r2);
#pragma omp parallel for num_threads(g->threads) schedule(static)
  for (size_t i = 0; i < nn; ++i) w->r3[i] = (w->r3[i] - w->r1[i] * w->r2[i]) / n4;
  r2c(g, w->r3, c);
}

static double powi(double x, int k) {
  if (k == 0) return 1.0;
  unsigned e = k < 0 ? (unsigned)(-k) : (unsigned)k;
  double r = 1.0, b = x;
  for (;;) {
    if (e & 1u) r *= b;
    e >>= 1;
    if (!e) break;
    b *= b;
  }
  return k < 0 ? 1.0 / r : r;
}

typedef struct {
  double nu, hnu, nuv, hnuv, omega, cfl;
  int nn, mm, nnv, mmv;
} coefs;

/* CFL_condition (:840-899), including the unused vz maximum */
static double cfl_dt(grid* g, work* w, const cplx* ps, const cplx* vz, const coefs* cf) {
  const size_t nn = (size_t)g->n * g->n;
  const double kcut = (double)g->n / 3.0, nrm = (double)g->n * g->n;
  derivk2(g, ps, w->c1, 1);
  derivk2(g, ps, w->c2, 2);
  c2r(g, w->c1, w->r1);
  c2r(g, w->c2, w->r2);
  double m = 0.0;
#pragma omp parallel for num_threads(g->threads) reduction(max : m) schedule(static)
  for (size_t i = 0; i < nn; ++i) {
    const double v = w->r1[i] * w->r1[i] + w->r2[i] * w->r2[i];
    if (v > m) m = v;
  }
  derivk2(g, vz, w->c1, 0);
  c2r(g, w->c1, w->r1);
  double mv = 0.0;
#pragma omp parallel for num_threads(g->threads) reduction(max : mv) schedule(static)
  for (size_t i = 0; i < nn; ++i) {
    const double v = w->r1[i] * w->r1[i];
    if (v > mv) mv = v;
  }
  (void)mv;
  const double tmp = sqrt(m) / nrm;
  return cf->cfl / (kcut * tmp + cf->nu * powi(kcut, 2 * cf->nn) + cf->nuv * powi(kcut, 2 * cf->nnv) + 2 * cf->omega);
}

/* RK step of order 4 (Rot2D3C.para.f90:545-611) */
static void rk_step(grid* g, work* w, cplx* ps, cplx* vz, const cplx* fp, const cplx* fz, double dt,
                    const coefs* cf, cplx* C1, cplx* C2, cplx* C3, cplx* C4, cplx* C5, cplx* C6) {
  const int n = g->n;
  const size_t S = (size_t)g->nh * n;
  memcpy(C1, ps, sizeof(cplx) * S);
  memcpy(C2, vz, sizeof(cplx) * S);
  for (int o = 4; o >= 1; --o) {
    laplak2(g, C1, C4);
    poisson(g, w, C1, C4, C5);
    poisson(g, w, C1, C2, C6);
    derivk2(g, C1, C3, 2);
    derivk2(g, C2, C4, 2);
#pragma omp parallel for num_threads(g->threads) schedule(static)
    for (int i = 0; i < g->nh; ++i)
      for (int j = 0; j < n; ++j) {
        const size_t id = (size_t)i * n + j;
        const double k2 = ka2(g, i, j);
        if (k2 <= g->kmax && k2 > g->tiny) {
          const double tmp1 = dt / (double)o, tmp2 = 1.0 / k2;
          double tmp3 = 1.0 + (cf->nu * powi(k2, cf->nn) + cf->hnu * powi(tmp2, cf->mm)) * tmp1;
          const double w2 = 2 * cf->omega;
          cplx a;
          a.re = (ps[id].re + ((-C5[id].re + w2 * C4[id].re) * tmp2 + fp[id].re) * tmp1) / tmp3;
          a.im = (ps[id].im + ((-C5[id].im + w2 * C4[id].im) * tmp2 + fp[id].im) * tmp1) / tmp3;
          tmp3 = 1.0 + (cf->nuv * powi(k2, cf->nnv) + cf->hnuv * powi(tmp2, cf->mmv)) * tmp1;
          cplx b;
          b.re = (vz[id].re + (C6[id].re + w2 * C3[id].re + fz[id].re) * tmp1) / tmp3;
          b.im = (vz[id].im + (C6[id].im + w2 * C3[id].im + fz[id].im) * tmp1) / tmp3;
          C1[id] = a;
          C2[id] = b;
        } else {
          C1[id].re = C1[id].im = 0.0;
          C2[id].re = C2[id].im = 0.0;
        }
      }
  }
  derivk2(g, C1, ps, 0);
  derivk2(g, C2, vz, 0);
}

/*
 * Run nsteps of the main loop body: optional CFL time step (cfl_mode != 0,
 * Rot2D3C.para.f90:399) then the RK step; the forcing is held fixed.
 * Arrays are the reference layouts (interleaved complex).  Returns the last
 * dt, or -1 on allocation failure.
 */
double r2d3c_cpu_run(int n, int threads, double* ps, double* vz, const double* fp, const double* fz,
                     int nsteps, int cfl_mode, double cfl_or_dt, double nu, double hnu, int nn_, int mm,
                     double nuv, double hnuv, int nnv, int mmv, double omega) {
  grid g;
  grid_init(&g, n, threads > 0 ? threads : 1);
  const size_t S = (size_t)g.nh * n, R = (size_t)n * n;
  work w;
  w.c1 = (cplx*)malloc(sizeof(cplx) * S);
  w.c2 = (cplx*)malloc(sizeof(cplx) * S);
  w.r1 = (double*)malloc(sizeof(double) * R);
  w.r2 = (double*)malloc(sizeof(double) * R);
  w.r3 = (double*)malloc(sizeof(double) * R);
  cplx* C[6];
  for (int i = 0; i < 6; ++i) C[i] = (cplx*)malloc(sizeof(cplx) * S);
  int ok = w.c1 && w.c2 && w.r1 && w.r2 && w.r3;
  for (int i = 0; i < 6; ++i) ok = ok && C[i];
  double dt = cfl_or_dt;
  if (ok) {
    coefs cf = {nu, hnu, nuv, hnuv, omega, cfl_or_dt, nn_, mm, nnv, mmv};
    for (int s = 0; s < nsteps; ++s) {
      if (cfl_mode) dt = cfl_dt(&g, &w, (const cplx*)ps, (const cplx*)vz, &cf);
      rk_step(&g, &w, (cplx*)ps, (cplx*)vz, (const cplx*)fp, (const cplx*)fz, dt, &cf, C[0], C[1], C[2],
              C[3], C[4], C[5]);
    }
  }
  free(w.c1);
  free(w.c2);
  free(w.r1);
  free(w.r2);
  free(w.r3);
  for (int i = 0; i < 6; ++i) free(C[i]);
  grid_free(&g);
  return ok ? dt : -1.0;
}

/* Standalone transforms (for the cross-check against the NumPy oracle). */
int r2d3c_cpu_r2c(int n, int threads, const double* in, double* out) {
  grid g;
  grid_init(&g, n, threads > 0 ? threads : 1);
  r2c(&g, in, (cplx*)out);
  grid_free(&g);
  return 0;
}

int r2d3c_cpu_c2r(int n, int threads, const double* in, double* out) {
  grid g;
  grid_init(&g, n, threads > 0 ? threads : 1);
  c2r(&g, (const cplx*)in, out);
  grid_free(&g);
  return 0;
}

int r2d3c_cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
