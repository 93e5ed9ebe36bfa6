/*
 * lbm_oracle.c -- CPU restatement of the lbmminiapp collide-stream hot path.
 *
 * TEST INFRASTRUCTURE (the oracle).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm may load it, and only as the
 * checker or the timed CPU baseline; the product library never calls it.
 *
 * It restates, in plain C with the reference's own data structures, the
 * single-rank CPU path of lbmminiapp:
 *
 *   - fluid-only compact storage with an adjacency list (int32 like the
 *     reference while Q * nFluid fits, int64 beyond) built with the
 *     semantics of GeometryAAAB::setupAdjacency
 *     (src/geometries/GeometryAAAB.cpp:18-124): neighbour x+c_s for AB push,
 *     x-c_s for AA and AB pull (:44-55); a wall or out-of-box neighbour maps
 *     to the own cell's opp(s) slot (:69-84); periodic axes wrap (:56-66, x
 *     only in the reference on one rank -- here every axis flagged periodic);
 *   - SOA slot index nFluid*s + i;
 *   - the BGK + Guo collision of KernelAA_SOA_Base::timestepEvenForce
 *     (src/kernels/KernelAA_SOA_Base.cpp:173-254), written with the same
 *     operation order and association so that, compiled without FMA
 *     contraction, it reproduces the reference Base kernels bit for bit;
 *   - AA even / odd (KernelAA_SOA_Base.cpp:173-254 / :257-342), AB push
 *     (KernelAB_SOA_Base.cpp:111-186), AB pull (KernelAB_SOA_Pull.cpp:113-194);
 *   - compat_rest_weight: the Q19 AA Unroll kernels weight the rest
 *     population's forcing term with 1/36 instead of 1/3
 *     (src/kernels/KernelAA_SOA_Unroll.cpp:556,770); setting the flag
 *     reproduces that.
 *
 * Extensions with no reference counterpart (parity for them is unpinned
 * against the reference; they are pinned by conservation / symmetry tests):
 *   - per-cell body force: F(x) = force + force_field(x);
 *   - porosity s(x) in [0,1], partial bounce-back after the collision
 *     (Walsh, Burwinkle & Saar 2009): post_s = (1-s) C_s(f) + s f_opp(s).
 *
 * Layout of every dense array exchanged with callers: cell index
 * c = x + nx*(y + ny*z); per-direction arrays are planar [q][c].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAXQ 27

/* Velocity sets in the reference's order and opposite table
 * (src/lattices/LatticeD3Q19.cpp:5-88, LatticeD3Q27.cpp:5-120). */
static const int Q19_C[19][3] = {
   {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
   {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0},
   {-1, 0, 1}, {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
   {0, 0, 0}};
static const int Q19_OPP[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};

static const int Q27_C[27][3] = {
   {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
   {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0},
   {-1, 0, 1}, {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
   {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1},
   {-1, -1, 1}, {-1, -1, -1}, {0, 0, 0}};
static const int Q27_OPP[27] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16,
                                15, 14, 25, 24, 23, 22, 21, 20, 19, 18, 26};

typedef struct {
   int Q;
   double c[ORACLE_MAXQ][3]; /* stencil as doubles, like the kernels' stencil_ */
   double w[ORACLE_MAXQ];
   double wf[ORACLE_MAXQ];   /* weight of the forcing term (compat flag) */
   int opp[ORACLE_MAXQ];
} oracle_lattice;

static int lattice_init(oracle_lattice* L, int Q, int compat_rest_weight)
{
   L->Q = Q;
   for (int s = 0; s < Q; s++) {
      const int* c = (Q == 19) ? Q19_C[s] : Q27_C[s];
      for (int d = 0; d < 3; d++) L->c[s][d] = (double)c[d];
      L->opp[s] = (Q == 19) ? Q19_OPP[s] : Q27_OPP[s];
      int n2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
      if (Q == 19) L->w[s] = n2 == 0 ? 1.0 / 3.0 : (n2 == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
      else L->w[s] = n2 == 0 ? 8.0 / 27.0 : (n2 == 1 ? 2.0 / 27.0 : (n2 == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
      L->wf[s] = L->w[s];
      if (compat_rest_weight && Q == 19 && n2 == 0) L->wf[s] = 1.0 / 36.0;
   }
   return (Q == 19 || Q == 27) ? 0 : 1;
}

/* One cell: BGK + Guo with the operation order of
 * KernelAA_SOA_Base.cpp:186-247; then optional partial bounce-back. */
static inline void collide_cell(const oracle_lattice* L, const double* d, double* out,
                                double omega, const double* F, double sp)
{
   const int Q = L->Q;
   double rho = 0.0;
   double v[3] = {0.0, 0.0, 0.0};
   for (int s = 0; s < Q; s++) {
      rho += d[s];
      v[0] += d[s] * L->c[s][0];
      v[1] += d[s] * L->c[s][1];
      v[2] += d[s] * L->c[s][2];
   }
   v[0] += 0.5 * F[0];
   v[1] += 0.5 * F[1];
   v[2] += 0.5 * F[2];
   double invRho = 1.0 / rho;
   v[0] *= invRho;
   v[1] *= invRho;
   v[2] *= invRho;
   double vdotv = 3.0 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
   double fdotv = 3.0 * (F[0] * v[0] + F[1] * v[1] + F[2] * v[2]);
   for (int s = 0; s < Q; s++) {
      double cdotv = 3.0 * (L->c[s][0] * v[0] + L->c[s][1] * v[1] + L->c[s][2] * v[2]);
      double cdotf = 3.0 * (L->c[s][0] * F[0] + L->c[s][1] * F[1] + L->c[s][2] * F[2]);
      double eq = L->w[s] * rho * (1.0 + cdotv + 0.5 * cdotv * cdotv - 0.5 * vdotv);
      double fdist = L->wf[s] * (cdotf - fdotv + cdotv * cdotf);
      out[s] = (1.0 - omega) * d[s] + omega * eq + (1.0 - 0.5 * omega) * fdist;
   }
   if (sp != 0.0) {
      double post[ORACLE_MAXQ];
      for (int s = 0; s < Q; s++) post[s] = (1.0 - sp) * out[s] + sp * d[L->opp[s]];
      for (int s = 0; s < Q; s++) out[s] = post[s];
   }
}

typedef struct {
   oracle_lattice L;
   int pattern; /* 0 AA, 1 AB push, 2 AB pull */
   int64_t nFluid;
   int64_t* fluidCell; /* dense cell index of each fluid point */
   int64_t* adj;       /* [Q][nFluid] slot indices (used when adj32 is NULL) */
   int32_t* adj32;     /* the same as int32, as the reference stores it, when Q*nFluid < 2^31 */
   double omega;
   double force[3];
   const double* forceField; /* planar [3][ncell] or NULL */
   const double* porosity;   /* [ncell] or NULL */
   int64_t ncell;
} oracle_state;

static int build_state(oracle_state* S, int Q, int pattern, int compat, int nx, int ny, int nz,
                       const int* periodic, const unsigned char* solid)
{
   if (lattice_init(&S->L, Q, compat)) return 1;
   S->pattern = pattern;
   const int64_t ncell = (int64_t)nx * ny * nz;
   S->ncell = ncell;
   int64_t* fluidIdx = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
   if (!fluidIdx) return 2;
   int64_t nf = 0;
   for (int64_t c = 0; c < ncell; c++) fluidIdx[c] = (solid && solid[c]) ? -1 : nf++;
   S->nFluid = nf;
   S->fluidCell = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nf > 0 ? nf : 1));
   S->adj = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nf > 0 ? nf : 1) * Q);
   if (!S->fluidCell || !S->adj) { free(fluidIdx); return 2; }
   for (int64_t c = 0; c < ncell; c++)
      if (fluidIdx[c] >= 0) S->fluidCell[fluidIdx[c]] = c;
   const int dims[3] = {nx, ny, nz};
   const int push = (pattern == 1);
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      int64_t c = S->fluidCell[i];
      int p[3] = {(int)(c % nx), (int)((c / nx) % ny), (int)(c / ((int64_t)nx * ny))};
      for (int s = 0; s < Q; s++) {
         int dir = push ? s : S->L.opp[s];
         int nb[3];
         int inside = 1;
         for (int d = 0; d < 3; d++) {
            nb[d] = p[d] + (int)S->L.c[dir][d];
            if (!periodic || periodic[d]) {
               if (nb[d] < 0) nb[d] += dims[d];
               else if (nb[d] >= dims[d]) nb[d] -= dims[d];
            }
            if (nb[d] < 0 || nb[d] >= dims[d]) inside = 0;
         }
         int64_t nbf = -1;
         if (inside) nbf = fluidIdx[nb[0] + (int64_t)nx * (nb[1] + (int64_t)ny * nb[2])];
         S->adj[(int64_t)s * nf + i] = (nbf < 0) ? (int64_t)S->L.opp[s] * nf + i : (int64_t)s * nf + nbf;
      }
   }
   free(fluidIdx);
   if ((int64_t)Q * nf < 2147483647LL) {
      S->adj32 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1) * Q);
      if (!S->adj32) return 2;
      for (int64_t k = 0; k < (int64_t)Q * nf; k++) S->adj32[k] = (int32_t)S->adj[k];
      free(S->adj);
      S->adj = NULL;
   }
   return 0;
}

#define ADJ(S, k) ((S)->adj32 ? (int64_t)(S)->adj32[k] : (S)->adj[k])

static inline void cell_params(const oracle_state* S, int64_t i, double* F, double* sp)
{
   int64_t c = S->fluidCell[i];
   F[0] = S->force[0];
   F[1] = S->force[1];
   F[2] = S->force[2];
   if (S->forceField) {
      F[0] += S->forceField[c];
      F[1] += S->forceField[S->ncell + c];
      F[2] += S->forceField[2 * S->ncell + c];
   }
   *sp = S->porosity ? S->porosity[c] : 0.0;
}

/* AA even: read own slot opp(s), write own slot s (KernelAA_SOA_Base.cpp:173-254). */
static void aa_even(const oracle_state* S, double* f)
{
   const int Q = S->L.Q;
   const int64_t nf = S->nFluid;
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      double d[ORACLE_MAXQ], o[ORACLE_MAXQ], F[3], sp;
      cell_params(S, i, F, &sp);
      for (int s = 0; s < Q; s++) d[s] = f[(int64_t)S->L.opp[s] * nf + i];
      collide_cell(&S->L, d, o, S->omega, F, sp);
      for (int s = 0; s < Q; s++) f[(int64_t)s * nf + i] = o[s];
   }
}

/* AA odd: gather through the adjacency, scatter to loc[opp(s)]
 * (KernelAA_SOA_Base.cpp:257-342). */
static void aa_odd(const oracle_state* S, double* f)
{
   const int Q = S->L.Q;
   const int64_t nf = S->nFluid;
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      double d[ORACLE_MAXQ], o[ORACLE_MAXQ], F[3], sp;
      int64_t loc[ORACLE_MAXQ];
      cell_params(S, i, F, &sp);
      for (int s = 0; s < Q; s++) {
         loc[s] = ADJ(S, (int64_t)s * nf + i);
         d[s] = f[loc[s]];
      }
      collide_cell(&S->L, d, o, S->omega, F, sp);
      for (int s = 0; s < Q; s++) f[loc[S->L.opp[s]]] = o[s];
   }
}

/* AB push: own cell from src, scatter through the adjacency into tgt
 * (KernelAB_SOA_Base.cpp:111-186). */
static void ab_push(const oracle_state* S, const double* src, double* tgt)
{
   const int Q = S->L.Q;
   const int64_t nf = S->nFluid;
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      double d[ORACLE_MAXQ], o[ORACLE_MAXQ], F[3], sp;
      cell_params(S, i, F, &sp);
      for (int s = 0; s < Q; s++) d[s] = src[(int64_t)s * nf + i];
      collide_cell(&S->L, d, o, S->omega, F, sp);
      for (int s = 0; s < Q; s++) tgt[ADJ(S, (int64_t)s * nf + i)] = o[s];
   }
}

/* AB pull: gather through the adjacency from src, own cell into tgt
 * (KernelAB_SOA_Pull.cpp:113-194). */
static void ab_pull(const oracle_state* S, const double* src, double* tgt)
{
   const int Q = S->L.Q;
   const int64_t nf = S->nFluid;
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      double d[ORACLE_MAXQ], o[ORACLE_MAXQ], F[3], sp;
      cell_params(S, i, F, &sp);
      for (int s = 0; s < Q; s++) d[s] = src[ADJ(S, (int64_t)s * nf + i)];
      collide_cell(&S->L, d, o, S->omega, F, sp);
      for (int s = 0; s < Q; s++) tgt[(int64_t)s * nf + i] = o[s];
   }
}

static double now_seconds(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int lbm_oracle_max_threads(void)
{
#ifdef _OPENMP
   return omp_get_max_threads();
#else
   return 1;
#endif
}

typedef struct {
   oracle_state S;
   double* a;
   double* b;
   int64_t t;
   int cur; /* AB: 0 -> a holds the latest state, 1 -> b */
} oracle_run_state;

void lbm_oracle_destroy(void* handle)
{
   oracle_run_state* R = (oracle_run_state*)handle;
   if (!R) return;
   free(R->a);
   free(R->b);
   free(R->S.fluidCell);
   free(R->S.adj);
   free(R->S.adj32);
   free(R);
}

/*
 * Build the fluid list and adjacency and place the initial populations.
 * Q: 19 | 27.  pattern: 0 AA, 1 AB push, 2 AB pull.
 * f_init: logical populations (direction s of each cell), planar [Q][ncell];
 *         placed as the reference's initialize() places them: AA in slot
 *         opp(s) (PropagationAA.cpp:104-116), AB in slot s of both buffers
 *         (PropagationAB.cpp:130-143).  force_field / porosity must outlive
 *         the handle.  nthreads <= 0 keeps the OpenMP default.
 * Returns NULL on bad arguments or allocation failure.
 */
void* lbm_oracle_create(int Q, int pattern, int compat_rest_weight, int nx, int ny, int nz,
                        const int* periodic, const unsigned char* solid, double omega,
                        const double* force, const double* force_field, const double* porosity,
                        const double* f_init, int nthreads)
{
   if (nx <= 0 || ny <= 0 || nz <= 0 || pattern < 0 || pattern > 2) return NULL;
#ifdef _OPENMP
   if (nthreads > 0) omp_set_num_threads(nthreads);
#else
   (void)nthreads;
#endif
   oracle_run_state* R = (oracle_run_state*)calloc(1, sizeof(oracle_run_state));
   if (!R) return NULL;
   oracle_state* S = &R->S;
   if (build_state(S, Q, pattern, compat_rest_weight, nx, ny, nz, periodic, solid)) {
      lbm_oracle_destroy(R);
      return NULL;
   }
   S->omega = omega;
   for (int d = 0; d < 3; d++) S->force[d] = force ? force[d] : 0.0;
   S->forceField = force_field;
   S->porosity = porosity;
   const int64_t nf = S->nFluid;
   const int64_t ncell = S->ncell;
   R->a = (double*)malloc(sizeof(double) * (size_t)(nf > 0 ? nf : 1) * Q);
   R->b = (double*)malloc(sizeof(double) * (size_t)(nf > 0 ? nf : 1) * Q);
   if (!R->a || !R->b) {
      lbm_oracle_destroy(R);
      return NULL;
   }
#pragma omp parallel for schedule(static)
   for (int64_t i = 0; i < nf; i++) {
      int64_t c = S->fluidCell[i];
      for (int s = 0; s < Q; s++) {
         double v = f_init[(int64_t)s * ncell + c];
         if (pattern == 0) {
            R->a[(int64_t)S->L.opp[s] * nf + i] = v;
         } else {
            R->a[(int64_t)s * nf + i] = v;
            R->b[(int64_t)s * nf + i] = v;
         }
      }
   }
   return R;
}

/* Advance nsteps; seconds = wall time of the loop. */
int lbm_oracle_step(void* handle, int nsteps, double* seconds)
{
   oracle_run_state* R = (oracle_run_state*)handle;
   if (!R || nsteps < 0) return 1;
   double t0 = now_seconds();
   for (int k = 0; k < nsteps; k++) {
      if (R->S.pattern == 0) {
         if (R->t % 2 == 0) aa_even(&R->S, R->a);
         else aa_odd(&R->S, R->a);
      } else {
         double* src = R->cur ? R->b : R->a;
         double* tgt = R->cur ? R->a : R->b;
         if (R->S.pattern == 1) ab_push(&R->S, src, tgt);
         else ab_pull(&R->S, src, tgt);
         R->cur = 1 - R->cur;
      }
      R->t++;
   }
   if (seconds) *seconds = now_seconds() - t0;
   return 0;
}

long long lbm_oracle_fluid_count(void* handle)
{
   oracle_run_state* R = (oracle_run_state*)handle;
   return R ? (long long)R->S.nFluid : -1;
}

/* Raw slot buffer the reference would read back (AA: the single buffer; AB:
 * the buffer holding the latest step, i.e. dstrb_ after the swap in
 * src/propagation/PropagationAB.cpp:182-188), planar [Q][ncell], NaN at solid
 * cells. */
int lbm_oracle_read(void* handle, double* f_raw)
{
   oracle_run_state* R = (oracle_run_state*)handle;
   if (!R || !f_raw) return 1;
   const int Q = R->S.L.Q;
   const int64_t nf = R->S.nFluid, ncell = R->S.ncell;
   const double* src = (R->S.pattern != 0 && R->cur) ? R->b : R->a;
   const double nan = NAN;
   for (int64_t k = 0; k < (int64_t)Q * ncell; k++) f_raw[k] = nan;
   for (int64_t i = 0; i < nf; i++) {
      int64_t c = R->S.fluidCell[i];
      for (int s = 0; s < Q; s++) f_raw[(int64_t)s * ncell + c] = src[(int64_t)s * nf + i];
   }
   return 0;
}

/* create + step + read + destroy.  Returns 0 on success, 1 for bad
 * arguments or allocation failure. */
int lbm_oracle_run(int Q, int pattern, int compat_rest_weight, int nx, int ny, int nz,
                   const int* periodic, const unsigned char* solid, double omega,
                   const double* force, const double* force_field, const double* porosity,
                   const double* f_init, int nsteps, int nthreads, double* f_raw,
                   double* seconds)
{
   if (nsteps < 0) return 1;
   void* R = lbm_oracle_create(Q, pattern, compat_rest_weight, nx, ny, nz, periodic, solid, omega,
                               force, force_field, porosity, f_init, nthreads);
   if (!R) return 1;
   int rc = lbm_oracle_step(R, nsteps, seconds);
   if (!rc) rc = lbm_oracle_read(R, f_raw);
   lbm_oracle_destroy(R);
   return rc;
}
