/*
 * ppfv_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of Sayram-2D's per-step hot path.
 *
 * This file is the checker, not the product. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it. The GPU library never calls it.
 *
 * It restates, in plain C and in the same arithmetic order, the reference's
 *   Solver::update_Lambda            source/Solver.cc:57-65
 *   Solver::fill_vertex_from_cells   source/Solver.cc:299-383
 *   Solver::fill_vertex_from_bcs     source/Solver.cc:385-422
 *   Solver::a_sigma_func             source/Solver.cc:68-97  (general formula with Edge geometry,
 *                                    Mesh.cc:67-155 / Edge.h:40-53)
 *   Solver::calculate_mu             source/Solver.h:63-67
 *   Solver::apply_inner_face_pair    source/Solver.cc:99-141
 *   Solver::apply_dirichlet_face     source/Solver.cc:143-164
 *   Solver::apply_boundary_faces     source/Solver.cc:204-267
 *   Solver::assemble                 source/Solver.cc:167-202 (diagonal + RHS, loss folded in)
 *   Eigen setFromTriplets            duplicates summed in triplet order (the order the loops
 *                                    above push them), reproduced by accumulating in loop order
 *   Solver::update                   source/Solver.cc:270-290 (solve + copy back K=j*nx+i -> (i,j))
 * with the direct sparse solve done by banded LU without pivoting (banded_lu.h).
 *
 * Layouts: per-cell fields are (nx, ny) alpha-major, index i*ny + j (xtensor row-major, as the
 * reference's Equation fields). The linear system is in the reference's system order
 * K = j*nx + i (Mesh.h:66-68). The matrix is returned as five diagonals of length N = nx*ny:
 *   M5[0*N+K] = M(K,K), M5[1*N+K] = M(K,K-1), M5[2*N+K] = M(K,K+1),
 *   M5[3*N+K] = M(K,K-nx), M5[4*N+K] = M(K,K+nx)      (0 where the neighbour does not exist)
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused (bit-exact against the
 * reference sources compiled the same way).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "banded_lu.h"

#define ORC_EPS DBL_EPSILON /* gEPS, source/common.h:38 */

enum { ORC_XMIN = 0, ORC_XMAX = 1, ORC_YMIN = 2, ORC_YMAX = 3 }; /* BCTypes.h:13 */
enum { ORC_DIRICHLET = 0, ORC_ZEROFLUX = 1 };                    /* BCTypes.h:16 */
enum { ORC_IM = 0, ORC_JP = 1, ORC_IP = 2, ORC_JM = 3 };         /* Mesh.h:76-79 */

typedef struct {
  int nx, ny;
  const double* x_edges; /* nx+1 */
  const double* y_edges; /* ny+1 */
  double dt;
  int bc[4];                                   /* XMIN, XMAX, YMIN, YMAX */
  const double *G, *Dxx, *Dxy, *Dyy, *inv_tau; /* alpha-major (nx, ny) */
  const double* dir[4]; /* Dirichlet vertex values: XMIN/XMAX indexed by j in [0,ny],
                           YMIN/YMAX indexed by i in [0,nx]; NULL for zero-flux sides */
} orc_problem;

typedef struct {
  const orc_problem* p;
  double* xc; /* cell centres x_(i) = 0.5*(xl+xr), Mesh.cc:50 */
  double* yc;
  double* dxc; /* widths, Mesh.cc:49 */
  double* dyc;
  double* L;  /* Lambda per cell: 4 doubles, row-major 2x2, alpha-major cell order */
  double* vf; /* vertex f, (nx+1, ny+1), index i*(ny+1)+j */
} orc_ws;

static int ws_init(orc_ws* w, const orc_problem* p) {
  const int nx = p->nx, ny = p->ny;
  memset(w, 0, sizeof(*w));
  w->p = p;
  w->xc = (double*)malloc(sizeof(double) * nx);
  w->yc = (double*)malloc(sizeof(double) * ny);
  w->dxc = (double*)malloc(sizeof(double) * nx);
  w->dyc = (double*)malloc(sizeof(double) * ny);
  w->L = (double*)malloc(sizeof(double) * 4 * (size_t)nx * ny);
  w->vf = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * (ny + 1));
  if (!w->xc || !w->yc || !w->dxc || !w->dyc || !w->L || !w->vf) return -1;
  for (int i = 0; i < nx; ++i) { /* Mesh::build_geometry_from_edges_, Mesh.cc:36-65 */
    const double xl = p->x_edges[i], xr = p->x_edges[i + 1];
    w->dxc[i] = xr - xl;
    w->xc[i] = 0.5 * (xl + xr);
  }
  for (int j = 0; j < ny; ++j) {
    const double yb = p->y_edges[j], yt = p->y_edges[j + 1];
    w->dyc[j] = yt - yb;
    w->yc[j] = 0.5 * (yb + yt);
  }
  /* Solver::update_Lambda, Solver.cc:57-65: Lambda = [[Dxx*G, Dxy*G],[Dxy*G, Dyy*G]] */
  for (size_t c = 0; c < (size_t)nx * ny; ++c) {
    w->L[4 * c + 0] = p->Dxx[c] * p->G[c];
    w->L[4 * c + 1] = p->Dxy[c] * p->G[c];
    w->L[4 * c + 2] = p->Dxy[c] * p->G[c];
    w->L[4 * c + 3] = p->Dyy[c] * p->G[c];
  }
  return 0;
}

static void ws_free(orc_ws* w) {
  free(w->xc); free(w->yc); free(w->dxc); free(w->dyc); free(w->L); free(w->vf);
}

static int check_problem(const orc_problem* p) {
  if (!p || p->nx < 1 || p->ny < 1 || !p->x_edges || !p->y_edges) return -1;
  if (!p->G || !p->Dxx || !p->Dxy || !p->Dyy || !p->inv_tau) return -1;
  for (int i = 0; i < p->nx; ++i) if (!(p->x_edges[i + 1] > p->x_edges[i])) return -1;
  for (int j = 0; j < p->ny; ++j) if (!(p->y_edges[j + 1] > p->y_edges[j])) return -1;
  for (int s = 0; s < 4; ++s) {
    if (p->bc[s] != ORC_DIRICHLET && p->bc[s] != ORC_ZEROFLUX) return -1;
    if (p->bc[s] == ORC_DIRICHLET && !p->dir[s]) return -2; /* Solver.cc:393 "missing value" */
  }
  return 0;
}

#define F(i, j) f[(size_t)(i) * ny + (j)]
#define VF(i, j) w->vf[(size_t)(i) * (ny + 1) + (j)]

static double lerp_(double x, double x0, double x1, double f0, double f1) { /* Solver.cc:304-310 */
  const double denom = (x1 - x0);
  if (denom == 0.0) return 0.5 * (f0 + f1);
  const double w0 = (x1 - x) / denom;
  const double w1 = (x - x0) / denom;
  return w0 * f0 + w1 * f1;
}

/* Solver::update_vertex_f = fill_vertex_from_cells + fill_vertex_from_bcs */
static void vertex_f(orc_ws* w, const double* f) {
  const orc_problem* p = w->p;
  const int nx = p->nx, ny = p->ny;
  const double* xe = p->x_edges;
  const double* ye = p->y_edges;
  /* corners, Solver.cc:314-319 */
  VF(0, 0) = F(0, 0);
  VF(nx, 0) = F(nx - 1, 0);
  VF(0, ny) = F(0, ny - 1);
  VF(nx, ny) = F(nx - 1, ny - 1);
  /* interior bilinear, Solver.cc:326-349 */
  for (int i = 1; i < nx; ++i) {
    for (int j = 1; j < ny; ++j) {
      const double xv = xe[i], yv = ye[j];
      const double xL = w->xc[i - 1], xR = w->xc[i];
      const double yB = w->yc[j - 1], yT = w->yc[j];
      const double denom_x = (xR - xL);
      const double denom_y = (yT - yB);
      const double wxL = (xR - xv) / denom_x;
      const double wxR = (xv - xL) / denom_x;
      const double wyB = (yT - yv) / denom_y;
      const double wyT = (yv - yB) / denom_y;
      VF(i, j) = wxL * wyB * F(i - 1, j - 1) + wxR * wyB * F(i, j - 1) + wxL * wyT * F(i - 1, j) +
                 wxR * wyT * F(i, j);
    }
  }
  /* vertical boundary edges, Solver.cc:355-365 */
  for (int j = 1; j < ny; ++j) {
    const double yv = ye[j], y0 = w->yc[j - 1], y1 = w->yc[j];
    VF(0, j) = lerp_(yv, y0, y1, F(0, j - 1), F(0, j));
    VF(nx, j) = lerp_(yv, y0, y1, F(nx - 1, j - 1), F(nx - 1, j));
  }
  /* horizontal boundary edges, Solver.cc:371-381 */
  for (int i = 1; i < nx; ++i) {
    const double xv = xe[i], x0 = w->xc[i - 1], x1 = w->xc[i];
    VF(i, 0) = lerp_(xv, x0, x1, F(i - 1, 0), F(i, 0));
    VF(i, ny) = lerp_(xv, x0, x1, F(i - 1, ny - 1), F(i, ny - 1));
  }
  /* Dirichlet overrides in the order XMIN, XMAX, YMIN, YMAX (later side wins at corners),
     Solver.cc:398-419 */
  if (p->bc[ORC_XMIN] == ORC_DIRICHLET)
    for (int j = 0; j <= ny; ++j) VF(0, j) = p->dir[ORC_XMIN][j];
  if (p->bc[ORC_XMAX] == ORC_DIRICHLET)
    for (int j = 0; j <= ny; ++j) VF(nx, j) = p->dir[ORC_XMAX][j];
  if (p->bc[ORC_YMIN] == ORC_DIRICHLET)
    for (int i = 0; i <= nx; ++i) VF(i, 0) = p->dir[ORC_YMIN][i];
  if (p->bc[ORC_YMAX] == ORC_DIRICHLET)
    for (int i = 0; i <= nx; ++i) VF(i, ny) = p->dir[ORC_YMAX][i];
}

/* Solver::a_sigma_func, Solver.cc:68-97, with the edge of cell (i,j) in direction inbr built
   as Mesh::build_connectivity_ does (Mesh.cc:80-151): vertices A = v(0), B = v(1), unit
   normal n and length |B - A|. */
static void a_sigma(const orc_ws* w, int i, int j, int inbr, double* aa, double* ab, double* asig) {
  const orc_problem* p = w->p;
  const int ny = p->ny;
  const double* xe = p->x_edges;
  const double* ye = p->y_edges;
  double Ax, Ay, Bx, By, n0, n1;
  int ai, aj, bi, bj;
  switch (inbr) {
    case ORC_IM: /* XNEG: A=(i,j+1), B=(i,j) */
      Ax = xe[i]; Ay = ye[j + 1]; Bx = xe[i]; By = ye[j]; n0 = -1.0; n1 = 0.0;
      ai = i; aj = j + 1; bi = i; bj = j; break;
    case ORC_JP: /* YPOS: A=(i+1,j+1), B=(i,j+1) */
      Ax = xe[i + 1]; Ay = ye[j + 1]; Bx = xe[i]; By = ye[j + 1]; n0 = 0.0; n1 = 1.0;
      ai = i + 1; aj = j + 1; bi = i; bj = j + 1; break;
    case ORC_IP: /* XPOS: A=(i+1,j), B=(i+1,j+1) */
      Ax = xe[i + 1]; Ay = ye[j]; Bx = xe[i + 1]; By = ye[j + 1]; n0 = 1.0; n1 = 0.0;
      ai = i + 1; aj = j; bi = i + 1; bj = j + 1; break;
    default: /* ORC_JM, YNEG: A=(i,j), B=(i+1,j) */
      Ax = xe[i]; Ay = ye[j]; Bx = xe[i + 1]; By = ye[j]; n0 = 0.0; n1 = -1.0;
      ai = i; aj = j; bi = i + 1; bj = j; break;
  }
  const double ex = Bx - Ax, ey = By - Ay;
  const double length = sqrt(ex * ex + ey * ey); /* Edge::set, Edge.h:43 */
  const double Kx = w->xc[i], Ky = w->yc[j];
  const double vkb0 = Bx - Kx, vkb1 = By - Ky;
  const double vka0 = Ax - Kx, vka1 = Ay - Ky;
  const double rvkb0 = vkb1, rvkb1 = -vkb0;
  const double rvka0 = vka1, rvka1 = -vka0;
  const double* L = &w->L[4 * ((size_t)i * ny + j)];
  /* n^T * Lambda (row vector), then dotted with the rotated vector */
  const double t0 = n0 * L[0] + n1 * L[2];
  const double t1 = n0 * L[1] + n1 * L[3];
  const double a_a = length * (t0 * rvkb0 + t1 * rvkb1) / (vka0 * rvkb0 + vka1 * rvkb1);
  const double a_b = length * (t0 * rvka0 + t1 * rvka1) / (vkb0 * rvka0 + vkb1 * rvka1);
  *aa = a_a;
  *ab = a_b;
  *asig = a_a * VF(ai, aj) + a_b * VF(bi, bj);
}

static int rinbr(int inbr) { return (inbr + 2) & 3; } /* Mesh.h:115 {2,3,0,1} */

/* vertex values at the A / B end of the edge of cell (i,j) in direction inbr (Mesh.cc:80-151) */
static double vfA_(const orc_ws* w, int i, int j, int inbr) {
  const int ny = w->p->ny;
  switch (inbr) {
    case ORC_IM: return VF(i, j + 1);
    case ORC_JP: return VF(i + 1, j + 1);
    case ORC_IP: return VF(i + 1, j);
    default: return VF(i, j);
  }
}
static double vfB_(const orc_ws* w, int i, int j, int inbr) {
  const int ny = w->p->ny;
  switch (inbr) {
    case ORC_IM: return VF(i, j);
    case ORC_JP: return VF(i, j + 1);
    case ORC_IP: return VF(i + 1, j + 1);
    default: return VF(i + 1, j);
  }
}

typedef struct {
  double* M5;
  double* R;
  long N;
  int nx;
  double* B5; /* optional: forward-error scale of every entry (same formulas on |terms|) */
} orc_sys;

/* add value v to diagonal d (0 = M(K,K), 1 = W, 2 = E, 3 = S, 4 = N) of row r */
static void add_entry(orc_sys* s, long r, int d, double v) { s->M5[(long)d * s->N + r] += v; }
static void add_bound(orc_sys* s, long r, int d, double v) {
  if (s->B5) s->B5[(long)d * s->N + r] += v;
}

/* Solver::apply_inner_face_pair, Solver.cc:99-141 */
static void inner_face_pair(const orc_ws* w, const double* f, orc_sys* s, int i, int j, int inbr) {
  const int nx = w->p->nx, ny = w->p->ny;
  double aaK, abK, aK, aaL, abL, aL;
  a_sigma(w, i, j, inbr, &aaK, &abK, &aK);
  int li = i, lj = j;
  if (inbr == ORC_IM) li = i - 1;
  else if (inbr == ORC_IP) li = i + 1;
  else if (inbr == ORC_JM) lj = j - 1;
  else lj = j + 1;
  a_sigma(w, li, lj, rinbr(inbr), &aaL, &abL, &aL);
  /* calculate_mu, Solver.h:63-67 */
  const double denom = fabs(aK) + fabs(aL) + 2 * ORC_EPS;
  const double muK = (fabs(aL) + ORC_EPS) / denom;
  const double muL = 1 - muK;
  const double B = muL * aL - muK * aK;
  const double Babs = fabs(B);
  const double Bp = (Babs + B) / 2.0;
  const double Bm = (Babs - B) / 2.0;
  const double AK = muK * (aaK + abK) + Bp / (F(i, j) + ORC_EPS);
  const double AL = muL * (aaL + abL) + Bm / (F(li, lj) + ORC_EPS);
  const long K = (long)j * nx + i, L = (long)lj * nx + li;
  if (s->B5) { /* every sum replaced by the sum of magnitudes of its terms */
    const int ny_ = w->p->ny;
    double tA, tB, tK, tL;
    (void)ny_;
    tA = tB = tK = tL = 0.0;
    double a0, a1, a2;
    a_sigma(w, i, j, inbr, &a0, &a1, &a2);
    (void)a2;
    tK = fabs(a0) * fabs(vfA_(w, i, j, inbr)) + fabs(a1) * fabs(vfB_(w, i, j, inbr));
    a_sigma(w, li, lj, rinbr(inbr), &a0, &a1, &a2);
    tL = fabs(a0) * fabs(vfA_(w, li, lj, rinbr(inbr))) + fabs(a1) * fabs(vfB_(w, li, lj, rinbr(inbr)));
    tA = muK * (fabs(aaK) + fabs(abK)) + (muL * tL + muK * tK) / (F(i, j) + ORC_EPS);
    tB = muL * (fabs(aaL) + fabs(abL)) + (muL * tL + muK * tK) / (F(li, lj) + ORC_EPS);
    const int dKL_ = (inbr == ORC_IM) ? 1 : (inbr == ORC_IP) ? 2 : (inbr == ORC_JM) ? 3 : 4;
    const int dLK_ = (dKL_ == 1) ? 2 : (dKL_ == 2) ? 1 : (dKL_ == 3) ? 4 : 3;
    add_bound(s, K, 0, tA);
    add_bound(s, K, dKL_, tB);
    add_bound(s, L, 0, tB);
    add_bound(s, L, dLK_, tA);
  }
  /* K's neighbour L lies west (inbr = im) or south (inbr = jm) of K */
  const int dKL = (inbr == ORC_IM) ? 1 : (inbr == ORC_IP) ? 2 : (inbr == ORC_JM) ? 3 : 4;
  const int dLK = (dKL == 1) ? 2 : (dKL == 2) ? 1 : (dKL == 3) ? 4 : 3;
  add_entry(s, K, 0, AK);
  add_entry(s, K, dKL, -AL);
  add_entry(s, L, 0, AL);
  add_entry(s, L, dLK, -AK);
}

/* Solver::apply_dirichlet_face, Solver.cc:143-164 */
static void dirichlet_face(const orc_ws* w, const double* f, orc_sys* s, int i, int j, int inbr) {
  const int nx = w->p->nx, ny = w->p->ny;
  double aa, ab, aK;
  a_sigma(w, i, j, inbr, &aa, &ab, &aK);
  const double B = -aK;
  const double Babs = fabs(B);
  const double Bp = (Babs + B) / 2.0;
  const double Bm = (Babs - B) / 2.0;
  const double AK = aa + ab + Bp / (F(i, j) + ORC_EPS);
  const long K = (long)j * nx + i;
  add_entry(s, K, 0, AK);
  add_bound(s, K, 0, fabs(aa) + fabs(ab) +
            (fabs(aa) * fabs(vfA_(w, i, j, inbr)) + fabs(ab) * fabs(vfB_(w, i, j, inbr))) / (F(i, j) + ORC_EPS));
  s->R[K] += Bm;
}

static void assemble_ws(const orc_ws* w, const double* f, double* M5, double* R, double* B5) {
  const orc_problem* p = w->p;
  const int nx = p->nx, ny = p->ny;
  const long N = (long)nx * ny;
  orc_sys s = {M5, R, N, nx, B5};
  memset(M5, 0, sizeof(double) * 5 * (size_t)N);
  if (B5) memset(B5, 0, sizeof(double) * 5 * (size_t)N);
  memset(R, 0, sizeof(double) * (size_t)N);
  /* 1) interior faces: west faces, then south faces (Solver.cc:172-182) */
  for (int i = 1; i < nx; ++i)
    for (int j = 0; j < ny; ++j) inner_face_pair(w, f, &s, i, j, ORC_IM);
  for (int i = 0; i < nx; ++i)
    for (int j = 1; j < ny; ++j) inner_face_pair(w, f, &s, i, j, ORC_JM);
  /* 2) boundary faces, XMIN, XMAX, YMIN, YMAX; zero-flux sides add nothing (Solver.cc:204-267) */
  if (p->bc[ORC_XMIN] == ORC_DIRICHLET)
    for (int j = 0; j < ny; ++j) dirichlet_face(w, f, &s, 0, j, ORC_IM);
  if (p->bc[ORC_XMAX] == ORC_DIRICHLET)
    for (int j = 0; j < ny; ++j) dirichlet_face(w, f, &s, nx - 1, j, ORC_IP);
  if (p->bc[ORC_YMIN] == ORC_DIRICHLET)
    for (int i = 0; i < nx; ++i) dirichlet_face(w, f, &s, i, 0, ORC_JM);
  if (p->bc[ORC_YMAX] == ORC_DIRICHLET)
    for (int i = 0; i < nx; ++i) dirichlet_face(w, f, &s, i, ny - 1, ORC_JP);
  /* 3) diagonal: UKK*(1+dt/tau) with UKK = G*dx*dy/dt, RHS += UKK*f (Solver.cc:190-199,
        Mesh.h:61-63) */
  for (int i = 0; i < nx; ++i) {
    for (int j = 0; j < ny; ++j) {
      const long K = (long)j * nx + i;
      const size_t c = (size_t)i * ny + j;
      const double UKK = p->G[c] * (w->dxc[i] * w->dyc[j] / p->dt);
      add_entry(&s, K, 0, UKK * (1 + p->dt * p->inv_tau[c]));
      add_bound(&s, K, 0, UKK * (1 + p->dt * p->inv_tau[c]));
      R[K] += UKK * F(i, j);
    }
  }
}

/* ---------------------------------------------------------------- exported API */

/* Vertex values of f (alpha-major) after the Dirichlet overrides; vf is (nx+1)*(ny+1). */
int orc_vertex_f(const orc_problem* p, const double* f, double* vf) {
  if (check_problem(p)) return -1;
  orc_ws w;
  if (ws_init(&w, p)) { ws_free(&w); return -3; }
  vertex_f(&w, f);
  memcpy(vf, w.vf, sizeof(double) * (size_t)(p->nx + 1) * (p->ny + 1));
  ws_free(&w);
  return 0;
}

/* One-sided face coefficients (a_sigma_A, a_sigma_B) and a_sigma of cell (i,j), direction inbr,
   with vertex values computed from f. */
int orc_face_coeffs(const orc_problem* p, const double* f, int i, int j, int inbr, double* out3) {
  if (check_problem(p) || i < 0 || j < 0 || i >= p->nx || j >= p->ny || inbr < 0 || inbr > 3)
    return -1;
  orc_ws w;
  if (ws_init(&w, p)) { ws_free(&w); return -3; }
  vertex_f(&w, f);
  a_sigma(&w, i, j, inbr, &out3[0], &out3[1], &out3[2]);
  ws_free(&w);
  return 0;
}

/* Assemble M (five diagonals, 5*N) and R (N) from f (alpha-major). */
int orc_assemble(const orc_problem* p, const double* f, double* M5, double* R) {
  int rc = check_problem(p);
  if (rc) return rc;
  orc_ws w;
  if (ws_init(&w, p)) { ws_free(&w); return -3; }
  vertex_f(&w, f);
  assemble_ws(&w, f, M5, R, NULL);
  ws_free(&w);
  return 0;
}

/* As orc_assemble, plus B5: for every entry the same expression evaluated on the magnitudes of
   its terms (sums of |products|), the scale of its floating-point rounding error. */
int orc_assemble_bound(const orc_problem* p, const double* f, double* M5, double* R, double* B5) {
  int rc = check_problem(p);
  if (rc) return rc;
  orc_ws w;
  if (ws_init(&w, p)) { ws_free(&w); return -3; }
  vertex_f(&w, f);
  assemble_ws(&w, f, M5, R, B5);
  ws_free(&w);
  return 0;
}

/* Direct solve of M x = R (system order) by banded LU without pivoting. */
int orc_solve(int nx, int ny, const double* M5, const double* R, double* x) {
  const long N = (long)nx * ny, p = nx, q = nx;
  double* band = (double*)calloc((size_t)N * (size_t)(p + q + 1), sizeof(double));
  if (!band) return -3;
  for (long K = 0; K < N; ++K) {
    band[blu_idx(K, K, p, q)] = M5[K];
    if (K - 1 >= 0 && nx > 1 && (K % nx) != 0) band[blu_idx(K, K - 1, p, q)] = M5[N + K];
    if (K + 1 < N && nx > 1 && (K % nx) != nx - 1) band[blu_idx(K, K + 1, p, q)] = M5[2 * N + K];
    if (K - nx >= 0) band[blu_idx(K, K - nx, p, q)] += M5[3 * N + K];
    if (K + nx < N) band[blu_idx(K, K + nx, p, q)] += M5[4 * N + K];
    /* for nx == 1 the W/E diagonals are empty and K-1 == K-nx: the += keeps S/N intact */
  }
  int rc = blu_factor(band, N, p, q);
  if (rc == 0) blu_solve(band, N, p, q, R, x);
  free(band);
  return rc;
}

/* nsteps backward-Euler steps of Solver::update (Solver.cc:270-290); f (alpha-major) is
   updated in place. Coefficients are time independent (Equation::update is a no-op in both
   reference cases). */
int orc_step(const orc_problem* p, double* f, int nsteps) {
  int rc = check_problem(p);
  if (rc) return rc;
  const int nx = p->nx, ny = p->ny;
  const long N = (long)nx * ny;
  orc_ws w;
  double* M5 = (double*)malloc(sizeof(double) * 5 * (size_t)N);
  double* R = (double*)malloc(sizeof(double) * (size_t)N);
  double* x = (double*)malloc(sizeof(double) * (size_t)N);
  if (ws_init(&w, p) || !M5 || !R || !x) { ws_free(&w); free(M5); free(R); free(x); return -3; }
  for (int s = 0; s < nsteps && rc == 0; ++s) {
    vertex_f(&w, f);
    assemble_ws(&w, f, M5, R, NULL);
    rc = orc_solve(nx, ny, M5, R, x);
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j) F(i, j) = x[(long)j * nx + i];
  }
  ws_free(&w);
  free(M5); free(R); free(x);
  return rc;
}

/* ---------------------------------------------------------------------------- D table
 * The Albert_Young cases build Dxx, Dxy, Dyy by bilinear interpolation in a table read from
 * HDF5 (Albert_Young_IO::read_D, Albert_Young_IO.cc:17-36), then convert the units:
 *   locate      Albert_Young.cc:94-110   position in a table assumed uniform in alpha0 and in
 *                                        log E, from the end points only
 *   calWeight   utils.h:44-58            weight of the lower node; beyond the last node the
 *                                        last node is used with weight 1
 *   interp2D    utils.h:24-41
 *   constructD  Albert_Young.cc:112-134  (the same in Albert_Young_LC.cc)
 *   e2p, dlogE_dp  utils.h:12-20;  gE0, gME, gC, gPI: common.h:38-43
 * The table's alpha0 axis is in degrees, as in the file (read_D converts it with * gPI / 180).
 * A position below the first node makes the reference convert a negative floor() to size_t,
 * which C++ leaves undefined; calWeight's own `i < 0` branch (first node, weight 1) states the
 * intent, and that is what is done here. */
typedef struct {
  int na, ne;                      /* nodes along alpha0 and E (both >= 2) */
  const double* alpha0_deg;        /* na: /alpha0 (degrees) */
  const double* E;                 /* ne: /E */
  const double *Daa, *Dap, *Dpp;   /* (na, ne) row-major: /Daa, /Dap, /Dpp */
} orc_dtable;

#define ORC_PI 3.141592653589793238462 /* gPI */
#define ORC_C 1.0                      /* gC */
#define ORC_E0 0.511875                /* gE0, MeV */

static double orc_e2p(double E, double E0) { return sqrt(E * (E + 2 * E0)) / ORC_C; }
static double orc_dlogE_dp(double logE, double E0) {
  const double E = exp(logE);
  return orc_e2p(E, ORC_E0) * ORC_C * ORC_C / (E * (E + E0));
}

static void orc_calweight(long* i, double* w, long n, double pos) {
  if (pos < 0.0) { /* see the note above */
    *i = 0;
    *w = 1.0;
  } else if (*i < n) {
    *w = 1.0 - (pos - (double)*i);
  } else {
    *i = n - 1;
    *w = 0.0;
  }
}

/* (nx, ny) alpha-major Dxx, Dxy, Dyy at the cell centres of the grid given by its edges. */
int orc_dtable_fields(int nx, int ny, const double* xe, const double* ye, const orc_dtable* t, double* Dxx,
                      double* Dxy, double* Dyy) {
  if (nx < 1 || ny < 1 || !t || t->na < 2 || t->ne < 2) return -1;
  const double xmin = t->alpha0_deg[0] * ORC_PI / 180, xmax = t->alpha0_deg[t->na - 1] * ORC_PI / 180;
  const double lymin = log(t->E[0]), lymax = log(t->E[t->ne - 1]);
  const double gme = ORC_E0 / (ORC_C * ORC_C);
  const double denorm = gme * gme * ORC_C * ORC_C;
  const double s2d = 3600 * 24;
  const long na1 = t->na - 1, ne1 = t->ne - 1;
  for (int i = 0; i < nx; ++i) {
    const double alpha0 = 0.5 * (xe[i] + xe[i + 1]);
    for (int j = 0; j < ny; ++j) {
      const double logE = 0.5 * (ye[j] + ye[j + 1]);
      const double p = orc_e2p(exp(logE), ORC_E0);
      const double px = (alpha0 - xmin) / (xmax - xmin) * (double)na1;
      const double py = (logE - lymin) / (lymax - lymin) * (double)ne1;
      long i0 = px >= 0.0 ? (long)floor(px) : 0, j0 = py >= 0.0 ? (long)floor(py) : 0;
      double wi, wj;
      orc_calweight(&i0, &wi, na1, px);
      orc_calweight(&j0, &wj, ne1, py);
      const double* raw[3] = {t->Daa, t->Dap, t->Dpp};
      double v[3];
      for (int k = 0; k < 3; ++k) {
        const double* r = raw[k];
        const long e = t->ne;
        v[k] = r[i0 * e + j0] * wi * wj + r[(i0 + 1) * e + j0] * (1 - wi) * wj +
               r[(i0 + 1) * e + j0 + 1] * (1 - wi) * (1 - wj) + r[i0 * e + j0 + 1] * wi * (1 - wj);
      }
      const long c = (long)i * ny + j;
      Dxx[c] = v[0] * denorm * s2d / (p * p);
      Dxy[c] = v[1] * denorm * s2d * orc_dlogE_dp(logE, ORC_E0) / p;
      Dyy[c] = v[2] * denorm * s2d * pow(orc_dlogE_dp(logE, ORC_E0), 2);
    }
  }
  return 0;
}
