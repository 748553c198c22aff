/*
 * bem_oracle.c -- CPU FP64 restatement of the full-3D Helmholtz collocation BEM.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the CUDA library
 * (libbemgpu.so).  It is imported only by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg, always as the checker, never as the product path.
 *
 * Discretisation (shared contract with the CUDA kernels, written independently):
 *   - one unknown per flat triangle, collocation at the centroid;
 *   - 7-point degree-5 triangle rule (Radon 1948; Stroud T2:5-1) for regular pairs;
 *   - near pairs (self panel, or centroid distance < eta * source-panel diameter):
 *     closed-form Laplace parts of S, D, K' and H on the flat triangle plus the
 *     bounded Helmholtz remainders by the same rule (21 points on the self panel,
 *     split at the centroid);
 *   - kernels G = exp(ikr)/(4 pi r), D = dG/dn_y, K' = dG/dn_x, H = d2G/dn_x dn_y
 *     (exp(-i w t) convention, numerics/helmholtz.jl:6-9 of the reference).
 *
 * Block algebra follows the reference:
 *   rigid / pressure release  M1 = 1/2 I - D - a H,  M2 = S + a (1/2 I + K')
 *     (solvers/bem/full.jl:104-127; a = i/k for Burton-Miller, full.jl:92, else 0).
 *     Rigid solves M1 x = M2 q_inc (full.jl:142-148); pressure release solves
 *     M2 x = M1 p_inc (full.jl:149-153).
 *   fluid Mueller  [I - De + Di, Se - g Si; -He + Hi/g, I + K'e - K'i] (full.jl:341)
 *   fluid CBIE     [1/2 I - De, Se; 1/2 I + Di, -g Si]                  (full.jl:344)
 *   incident traces p = exp(ik d.y), q = ik (d.n) p     (core/incident.jl:64-76)
 *   far field f(xh) = -(1/4pi) sum w (ik xh.n p + q) exp(-ik xh.y)  (full.jl:509-519)
 *
 * Parity pinned: against the reference's modal series (solvers/modal/sphere.jl) and the
 * amplitudes hard-coded in its own tests (see tests/golden/), not against the
 * reference's operators, which live in the third-party Inti.jl and cannot run here.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_PI 3.14159265358979323846
#define OR_INV4PI (1.0 / (4.0 * OR_PI))

/* Radon's 7-point rule: barycentric coordinates and weights (sum of weights = 1). */
static const double RW[7] = {
    0.225,
    0.13239415278850618074, 0.13239415278850618074, 0.13239415278850618074,
    0.12593918054482715260, 0.12593918054482715260, 0.12593918054482715260};
static const double RB[7][3] = {
    {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0},
    {0.05971587178976982046, 0.47014206410511508977, 0.47014206410511508977},
    {0.47014206410511508977, 0.05971587178976982046, 0.47014206410511508977},
    {0.47014206410511508977, 0.47014206410511508977, 0.05971587178976982046},
    {0.79742698535308732240, 0.10128650732345633880, 0.10128650732345633880},
    {0.10128650732345633880, 0.79742698535308732240, 0.10128650732345633880},
    {0.10128650732345633880, 0.10128650732345633880, 0.79742698535308732240}};

/* Panel geometry (one record per triangle). */
typedef struct {
  double v[3][3];  /* vertices in connectivity order */
  double c[3];     /* centroid = collocation point */
  double n[3];     /* unit normal (b-a)x(c-a) */
  double area;
  double diam;     /* longest edge */
  double g[7][3];  /* Gauss points */
} or_panel;

static inline double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void sub3(const double *a, const double *b, double *o) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
static inline void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* nodes: 3 x N column-major; tris: 3 x M column-major, 1-based (Gmsh order). */
int oracle_panels(const double *nodes, int64_t N, const int64_t *tris, int64_t M,
                  or_panel *out) {
  for (int64_t t = 0; t < M; ++t) {
    or_panel *p = &out[t];
    for (int a = 0; a < 3; ++a) {
      int64_t id = tris[3 * t + a] - 1;
      if (id < 0 || id >= N) return -1;
      for (int d = 0; d < 3; ++d) p->v[a][d] = nodes[3 * id + d];
    }
    double e1[3], e2[3], cr[3];
    sub3(p->v[1], p->v[0], e1);
    sub3(p->v[2], p->v[0], e2);
    cross3(e1, e2, cr);
    double len = sqrt(dot3(cr, cr));
    if (!(len > 0.0)) return -2;
    for (int d = 0; d < 3; ++d) {
      p->n[d] = cr[d] / len;
      p->c[d] = (p->v[0][d] + p->v[1][d] + p->v[2][d]) / 3.0;
    }
    p->area = 0.5 * len;
    double dm = 0.0;
    for (int a = 0; a < 3; ++a) {
      double e[3];
      sub3(p->v[(a + 1) % 3], p->v[a], e);
      double l = sqrt(dot3(e, e));
      if (l > dm) dm = l;
    }
    p->diam = dm;
    for (int q = 0; q < 7; ++q)
      for (int d = 0; d < 3; ++d)
        p->g[q][d] = RB[q][0] * p->v[0][d] + RB[q][1] * p->v[1][d] + RB[q][2] * p->v[2][d];
  }
  return 0;
}

/* Near test: self, or |c_i - c_j|^2 < eta^2 diam_j^2 (no fused multiply-add). */
static inline int is_near(const or_panel *P, int64_t i, int64_t j, double eta2) {
  if (i == j) return 1;
  double dx = P[i].c[0] - P[j].c[0];
  double dy = P[i].c[1] - P[j].c[1];
  double dz = P[i].c[2] - P[j].c[2];
  double d2 = dx * dx + dy * dy + dz * dz;
  double r2 = eta2 * (P[j].diam * P[j].diam);
  return d2 < r2;
}

/* CSR near list: rowptr[M+1], cols (capacity cap). Returns count or -1 if cap is short. */
int64_t oracle_near_pairs(const or_panel *P, int64_t M, double eta, int64_t *rowptr,
                          int64_t *cols, int64_t cap) {
  double eta2 = eta * eta;
  int64_t cnt = 0;
  for (int64_t i = 0; i < M; ++i) {
    rowptr[i] = cnt;
    for (int64_t j = 0; j < M; ++j) {
      if (is_near(P, i, j, eta2)) {
        if (cnt < cap) cols[cnt] = j;
        ++cnt;
      }
    }
  }
  rowptr[M] = cnt;
  return cnt > cap ? -1 : cnt;
}

/* ---- Helmholtz remainder functions (series for small z = k r) ---- */
/* E1(z) = e^{iz}(1 - iz) - 1 - z^2/2 = sum_{m>=3} (1-m)(iz)^m/m! */
/* E2(z) = e^{iz}(iz - 1) + 1         = sum_{m>=2} (m-1)(iz)^m/m! */
/* E3(z) = e^{iz}(3 - 3iz - z^2) - 3  = sum_{m>=2} (m-1)(m-3)(iz)^m/m! */
/* E0(z) = e^{iz} - 1                 = sum_{m>=1} (iz)^m/m! */
#define OR_SERIES_Z 0.5
static void remainders(double z, double complex *E0, double complex *E1,
                       double complex *E2, double complex *E3) {
  if (z < OR_SERIES_Z) {
    double complex t = 1.0, s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int m = 1; m <= 24; ++m) {
      t = t * (I * z) / (double)m; /* (iz)^m / m! */
      s0 += t;
      if (m >= 2) {
        s2 += (double)(m - 1) * t;
        s3 += (double)((m - 1) * (m - 3)) * t;
      }
      if (m >= 3) s1 += (double)(1 - m) * t;
    }
    *E0 = s0;
    *E1 = s1;
    *E2 = s2;
    *E3 = s3;
  } else {
    double complex e = cos(z) + I * sin(z);
    *E0 = e - 1.0;
    *E1 = e * (1.0 - I * z) - 1.0 - 0.5 * z * z;
    *E2 = e * (I * z - 1.0) + 1.0;
    *E3 = e * (3.0 - 3.0 * I * z - z * z) - 3.0;
  }
}

/* Full Helmholtz kernels at one source point (regular pairs). u = y - x. */
static void full_kernels(double k, const double *u, const double *nx, const double *ny,
                         double w, double complex *S, double complex *D,
                         double complex *K, double complex *H) {
  double r2 = dot3(u, u);
  double r = sqrt(r2);
  double z = k * r;
  double complex e = cos(z) + I * sin(z);
  double un_y = dot3(u, ny), un_x = dot3(u, nx), nn = dot3(nx, ny);
  double ir = 1.0 / r, ir3 = ir * ir * ir;
  double complex g = e * (OR_INV4PI * ir);
  double complex gp = e * (I * z - 1.0) * (OR_INV4PI * ir3); /* G'(r)/r */
  *S += w * g;
  *D += w * gp * un_y;
  *K -= w * gp * un_x;
  double c = un_x * un_y * ir * ir;
  *H += w * (e * OR_INV4PI * ir3) * ((1.0 - I * z) * nn - (3.0 - 3.0 * I * z - z * z) * c);
}

/* Remainder (Helmholtz minus Laplace, H also minus (k^2/2)(nx.ny) G0) at one point. */
static void rem_kernels(double k, const double *u, const double *nx, const double *ny,
                        double w, double complex *S, double complex *D,
                        double complex *K, double complex *H) {
  double r2 = dot3(u, u);
  double r = sqrt(r2);
  double z = k * r;
  double complex E0, E1, E2, E3;
  remainders(z, &E0, &E1, &E2, &E3);
  double un_y = dot3(u, ny), un_x = dot3(u, nx), nn = dot3(nx, ny);
  double ir = 1.0 / r, ir3 = ir * ir * ir;
  double c = un_x * un_y * ir * ir;
  *S += w * (OR_INV4PI * ir) * E0;
  *D += w * (OR_INV4PI * ir3) * E2 * un_y;
  *K -= w * (OR_INV4PI * ir3) * E2 * un_x;
  *H += w * (OR_INV4PI * ir3) * (E1 * nn - E3 * c);
}

/* Closed-form Laplace parts on a flat triangle: returns S0, D0, K0, H0 (real). */
static void laplace_parts(const or_panel *T, const double *x, const double *nx, int self,
                          double *S0, double *D0, double *K0, double *H0) {
  double Pint = 0.0, gP[3] = {0, 0, 0}, Hs = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double *Pa = T->v[a], *Pb = T->v[(a + 1) % 3];
    double e[3], s[3], m[3], w[3], wb[3], sw[3];
    sub3(Pb, Pa, e);
    double L = sqrt(dot3(e, e));
    for (int d = 0; d < 3; ++d) s[d] = e[d] / L;
    cross3(s, T->n, m);
    sub3(x, Pa, w);
    sub3(x, Pb, wb);
    double s0 = dot3(w, s);
    double sm = -s0, sp = L - s0;
    double t0 = -dot3(w, m);
    double dpl = dot3(w, T->n);
    double R02 = t0 * t0 + dpl * dpl; /* squared distance from x to the edge line */
    double Rm = sqrt(dot3(w, w)), Rp = sqrt(dot3(wb, wb));
    /* f = ln((Rp + sp)/(Rm + sm)) in a cancellation-free form per foot position */
    double f;
    if (sm >= 0.0)
      f = log((Rp + sp) / (Rm + sm));
    else if (sp <= 0.0)
      f = log((Rm - sm) / (Rp - sp));
    else
      f = log((Rp + sp) * (Rm - sm) / R02);
    Pint += t0 * f;
    for (int d = 0; d < 3; ++d) gP[d] -= m[d] * f;
    cross3(s, w, sw);
    double rho2 = dot3(sw, sw);
    if (rho2 > 1e-24 * L * L) Hs += dot3(nx, sw) / rho2 * (sp / Rp - sm / Rm);
  }
  double Om = 0.0, d = 0.0;
  if (!self) {
    double R0[3], R1[3], R2[3], t[3];
    sub3(T->v[0], x, R0);
    sub3(T->v[1], x, R1);
    sub3(T->v[2], x, R2);
    double r0 = sqrt(dot3(R0, R0)), r1 = sqrt(dot3(R1, R1)), r2 = sqrt(dot3(R2, R2));
    cross3(R1, R2, t);
    double num = dot3(R0, t);
    double den = r0 * r1 * r2 + dot3(R0, R1) * r2 + dot3(R0, R2) * r1 + dot3(R1, R2) * r0;
    Om = 2.0 * atan2(num, den);
    double xp[3];
    sub3(x, T->v[0], xp);
    d = dot3(xp, T->n);
  }
  *S0 = OR_INV4PI * (Pint + d * Om);
  *D0 = -OR_INV4PI * Om;
  *K0 = OR_INV4PI * (dot3(nx, gP) + dot3(nx, T->n) * Om);
  *H0 = -OR_INV4PI * Hs;
}

/* Operators of one panel pair (collocation point of panel i, source panel j). */
typedef struct {
  double complex S, D, K, H;
} or_ops;

static void pair_ops(const or_panel *P, int64_t i, int64_t j, int near, double k,
                     or_ops *o) {
  const double *x = P[i].c, *nx = P[i].n;
  const or_panel *T = &P[j];
  double complex S = 0, D = 0, K = 0, H = 0;
  if (!near) {
    for (int q = 0; q < 7; ++q) {
      double u[3];
      sub3(T->g[q], x, u);
      full_kernels(k, u, nx, T->n, RW[q] * T->area, &S, &D, &K, &H);
    }
  } else {
    int self = (i == j);
    double S0, D0, K0, H0;
    laplace_parts(T, x, nx, self, &S0, &D0, &K0, &H0);
    if (self) {
      double sa = T->area / 3.0;
      for (int a = 0; a < 3; ++a) {
        const double *Pa = T->v[a], *Pb = T->v[(a + 1) % 3];
        for (int q = 0; q < 7; ++q) {
          double y[3], u[3];
          for (int d = 0; d < 3; ++d)
            y[d] = RB[q][0] * T->c[d] + RB[q][1] * Pa[d] + RB[q][2] * Pb[d];
          sub3(y, x, u);
          rem_kernels(k, u, nx, T->n, RW[q] * sa, &S, &D, &K, &H);
        }
      }
    } else {
      for (int q = 0; q < 7; ++q) {
        double u[3];
        sub3(T->g[q], x, u);
        rem_kernels(k, u, nx, T->n, RW[q] * T->area, &S, &D, &K, &H);
      }
    }
    double nn = dot3(nx, T->n);
    S += S0;
    D += D0;
    K += K0;
    H += H0 + 0.5 * k * k * nn * S0;
  }
  o->S = S;
  o->D = D;
  o->K = K;
  o->H = H;
}

/* Exported for tests: the four operators of one pair, interleaved complex out[8]. */
void oracle_pair_ops(const or_panel *P, int64_t i, int64_t j, int near, double k,
                     double *out) {
  or_ops o;
  pair_ops(P, i, j, near, k, &o);
  out[0] = creal(o.S); out[1] = cimag(o.S);
  out[2] = creal(o.D); out[3] = cimag(o.D);
  out[4] = creal(o.K); out[5] = cimag(o.K);
  out[6] = creal(o.H); out[7] = cimag(o.H);
}

/* Exported for tests: closed-form Laplace parts at an arbitrary point. */
void oracle_laplace_parts(const or_panel *T, const double *x, const double *nx, int self,
                          double *out4) {
  laplace_parts(T, x, nx, self, &out4[0], &out4[1], &out4[2], &out4[3]);
}

/*
 * Rigid / pressure-release system operators, column-major n x n, interleaved complex.
 * M1 = 1/2 I - D - a H, M2 = S + a (1/2 I + K'), a = bm ? i/k : 0.
 */
int oracle_assemble_bm(const or_panel *P, int64_t n, double eta, double k, int bm,
                       double *M1, double *M2) {
  double eta2 = eta * eta;
  double complex a = bm ? I / k : 0.0;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      or_ops o;
      pair_ops(P, i, j, is_near(P, i, j, eta2), k, &o);
      double complex d = (i == j) ? 0.5 : 0.0;
      double complex m1 = d - o.D - a * o.H;
      double complex m2 = o.S + a * (d + o.K);
      int64_t idx = 2 * (i + j * n);
      M1[idx] = creal(m1);
      M1[idx + 1] = cimag(m1);
      M2[idx] = creal(m2);
      M2[idx + 1] = cimag(m2);
    }
  }
  return 0;
}

/*
 * The four raw operators S, D, K', H of every panel pair (target i, source j) at one
 * wavenumber, column-major n x n interleaved complex each.  The multi-region restatement
 * combines blocks of these (solvers/bem/regions.jl:189-236).
 */
int oracle_assemble_ops(const or_panel *P, int64_t n, double eta, double k, double *S,
                        double *D, double *K, double *H) {
  double eta2 = eta * eta;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      or_ops o;
      pair_ops(P, i, j, is_near(P, i, j, eta2), k, &o);
      int64_t idx = 2 * (i + j * n);
      S[idx] = creal(o.S); S[idx + 1] = cimag(o.S);
      D[idx] = creal(o.D); D[idx + 1] = cimag(o.D);
      K[idx] = creal(o.K); K[idx + 1] = cimag(o.K);
      H[idx] = creal(o.H); H[idx + 1] = cimag(o.H);
    }
  }
  return 0;
}

/*
 * Fluid system, column-major 2n x 2n interleaved complex.
 * formulation 0: Mueller, 1: CBIE.  k_int = k / h.
 */
int oracle_assemble_fluid(const or_panel *P, int64_t n, double eta, double k, double g,
                          double h, int formulation, double *A) {
  double eta2 = eta * eta;
  double ki = k / h;
  int64_t N = 2 * n;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) {
      int near = is_near(P, i, j, eta2);
      or_ops e, in;
      pair_ops(P, i, j, near, k, &e);
      pair_ops(P, i, j, near, ki, &in);
      double complex a11, a12, a21, a22;
      if (formulation == 0) {
        double complex d = (i == j) ? 1.0 : 0.0;
        a11 = d - e.D + in.D;
        a12 = e.S - g * in.S;
        a21 = -e.H + in.H / g;
        a22 = d + e.K - in.K;
      } else {
        double complex d = (i == j) ? 0.5 : 0.0;
        a11 = d - e.D;
        a12 = e.S;
        a21 = d + in.D;
        a22 = -g * in.S;
      }
      int64_t r1 = i, r2 = n + i, c1 = j, c2 = n + j;
      A[2 * (r1 + c1 * N)] = creal(a11); A[2 * (r1 + c1 * N) + 1] = cimag(a11);
      A[2 * (r1 + c2 * N)] = creal(a12); A[2 * (r1 + c2 * N) + 1] = cimag(a12);
      A[2 * (r2 + c1 * N)] = creal(a21); A[2 * (r2 + c1 * N) + 1] = cimag(a21);
      A[2 * (r2 + c2 * N)] = creal(a22); A[2 * (r2 + c2 * N) + 1] = cimag(a22);
    }
  }
  return 0;
}

/* Incident plane-wave traces at the collocation points (interleaved complex). */
void oracle_incident(const or_panel *P, int64_t n, double k, const double *dir, double *p,
                     double *q) {
  for (int64_t i = 0; i < n; ++i) {
    double ph = k * dot3(dir, P[i].c);
    double complex e = cos(ph) + I * sin(ph);
    double complex dq = I * k * dot3(dir, P[i].n) * e;
    p[2 * i] = creal(e);
    p[2 * i + 1] = cimag(e);
    q[2 * i] = creal(dq);
    q[2 * i + 1] = cimag(dq);
  }
}

/* Far-field amplitude for one observation direction (interleaved complex out[2]). */
void oracle_far_field(const or_panel *P, int64_t n, double k, const double *xhat,
                      const double *p, const double *q, double *out) {
  double complex tot = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    double complex pj = p[2 * j] + I * p[2 * j + 1];
    double complex qj = q[2 * j] + I * q[2 * j + 1];
    double complex a = I * k * dot3(xhat, P[j].n) * pj + qj;
    double complex s = 0.0;
    for (int g = 0; g < 7; ++g) {
      double ph = -k * dot3(xhat, P[j].g[g]);
      s += RW[g] * (cos(ph) + I * sin(ph));
    }
    tot += a * s * P[j].area;
  }
  tot = -tot * OR_INV4PI;
  out[0] = creal(tot);
  out[1] = cimag(tot);
}

int oracle_panel_size(void) { return (int)sizeof(or_panel); }

/*
 * Layer potentials of the surface traces at a point (fields/pressure.jl:448-471 of the
 * reference): exterior sum_j D_j p_j - S_j q_j, interior sum_j S_j q_j - D_j p_j, where
 * S_j, D_j are the unit-density single/double layers of panel j (7-point rule, or closed
 * form + remainder within eta diameters).  out[2] complex.
 */
void oracle_layer_potentials(const or_panel *P, int64_t n, double k, const double *x,
                             double eta, const double *p, const double *q, int interior,
                             double *out) {
  double complex acc = 0.0;
  const double zero[3] = {0.0, 0.0, 0.0};
  for (int64_t j = 0; j < n; ++j) {
    const or_panel *T = &P[j];
    double complex pj = p[2 * j] + I * p[2 * j + 1], qj = q[2 * j] + I * q[2 * j + 1];
    double dx = x[0] - T->c[0], dy = x[1] - T->c[1], dz = x[2] - T->c[2];
    double d2 = dx * dx + dy * dy + dz * dz;
    double lim = eta * T->diam;
    double complex S = 0, D = 0, K = 0, H = 0;
    if (d2 < lim * lim) {
      double S0, D0, K0, H0;
      laplace_parts(T, x, zero, 0, &S0, &D0, &K0, &H0);
      for (int g = 0; g < 7; ++g) {
        double u[3];
        sub3(T->g[g], x, u);
        rem_kernels(k, u, zero, T->n, RW[g] * T->area, &S, &D, &K, &H);
      }
      S += S0;
      D += D0;
    } else {
      for (int g = 0; g < 7; ++g) {
        double u[3];
        sub3(T->g[g], x, u);
        full_kernels(k, u, zero, T->n, RW[g] * T->area, &S, &D, &K, &H);
      }
    }
    acc += interior ? (S * qj - D * pj) : (D * pj - S * qj);
  }
  out[0] = creal(acc);
  out[1] = cimag(acc);
}

/* Sum of the panels' signed solid angles seen from x: 4 pi inside, 0 outside. */
double oracle_solid_angle(const or_panel *P, int64_t n, const double *x) {
  double om = 0.0;
  for (int64_t j = 0; j < n; ++j) {
    double R0[3], R1[3], R2[3], t[3];
    sub3(P[j].v[0], x, R0);
    sub3(P[j].v[1], x, R1);
    sub3(P[j].v[2], x, R2);
    double r0 = sqrt(dot3(R0, R0)), r1 = sqrt(dot3(R1, R1)), r2 = sqrt(dot3(R2, R2));
    cross3(R1, R2, t);
    double num = dot3(R0, t);
    double den = r0 * r1 * r2 + dot3(R0, R1) * r2 + dot3(R0, R2) * r1 + dot3(R1, R2) * r0;
    om += 2.0 * atan2(num, den);
  }
  return om;
}
