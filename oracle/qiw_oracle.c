/*
 * CPU oracle for the qMC diagram-integration path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C99 with complex FP64 arithmetic, the reference's
 * algorithm for one qMC integral of one topology group:
 *   - Sobol direction numbers and next!/skip!     src/scrambled_sobol.jl:66-208
 *   - Root / DoubleSimplexRoot transforms, J      src/qmc_integrate.jl:46,198-258,363-463
 *   - Sort / ExpModelFunction transforms          src/qmc_integrate.jl:99-165,282-334
 *   - contour_integral / qmc_integral             src/qmc_integrate.jl:497-507,565-612
 *   - TopologyEvaluator ctor + per-sample functor src/topology_eval.jl:249-437
 *   - _traverse_configuration_tree!               src/topology_eval.jl:454-556
 *   - LazyMatrixProduct push/pop/eval!            src/utility.jl:234-323
 *   - ExactAtomicPPGF interpolate!                src/exact_atomic_ppgf.jl:109-118
 * It deliberately follows the reference's recursion (not the DAG plan used by the CUDA
 * library), so the two are independent.  Only the tests, the smoke check and the
 * benchmark's CPU-baseline leg may call it.  The product library never links it.
 *
 * Threading: samples are split into contiguous ranges exactly like rank_sub_range
 * (src/mpi.jl:49-54, src/utility.jl:164-179) and each range is weighted by
 * length/N as in src/inchworm.jl:168-187; ranges are combined in rank order.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qiw_oracle.h"

typedef double complex cplx;

#define MAXN 32      /* max nodes in a configuration  */
#define MAXS 64      /* max sectors                    */
#define MAXD 16      /* max sector dimension            */
#define MAXP 64      /* max interaction pairs           */
#define MAXK 12      /* max order                        */

/* ------------------------------------------------------------------ Sobol */

int qiwo_sobol_directions(int D, const int64_t *poly, const int64_t *vinit, int vinit_cols,
                          uint32_t *m /* [D][32] */)
{
    for (int d = 0; d < D; ++d)
        for (int j = 0; j < 32; ++j) m[d * 32 + j] = 1u;
    for (int d = 2; d <= D; ++d) {
        uint32_t a = (uint32_t)poly[d - 1];
        int deg = 0;
        while ((a >> (deg + 1)) != 0) ++deg; /* floor(log2(a)) */
        uint32_t *md = m + (d - 1) * 32;
        for (int j = 0; j < deg; ++j) md[j] = (uint32_t)vinit[(d - 1) * vinit_cols + j];
        for (int j = deg + 1; j <= 32; ++j) {
            uint32_t ac = a;
            uint32_t v = md[j - deg - 1];
            for (int k = 0; k <= deg - 1; ++k) {
                v ^= ((ac & 1u) * md[j - deg + k - 1]) << (deg - k);
                ac >>= 1;
            }
            md[j - 1] = v;
        }
    }
    for (int j = 1; j <= 32; ++j)
        for (int d = 0; d < D; ++d) m[d * 32 + j - 1] *= (uint32_t)1u << (32 - j);
    return 0;
}

/* Sequential generator with the reference's next! semantics. */
typedef struct {
    int D;
    const uint32_t *m;
    uint32_t x[2 * MAXK + 2];
    uint32_t n;
} sobol_t;

static void sobol_init(sobol_t *s, int D, const uint32_t *m, const uint32_t *x0)
{
    s->D = D;
    s->m = m;
    for (int d = 0; d < D; ++d) s->x[d] = x0 ? x0[d] : 0u;
    s->n = 0;
}

static void sobol_next(sobol_t *s, double *x)
{
    if (s->n == 0) {
        s->n += 1;
        for (int d = 0; d < s->D; ++d) x[d] = ldexp((double)s->x[d], -32);
        return;
    }
    s->n += 1;
    uint32_t v = s->n - 1;
    int c = 0;
    while (!(v & 1u)) { v >>= 1; ++c; }
    for (int d = 0; d < s->D; ++d) {
        s->x[d] ^= s->m[d * 32 + c];
        x[d] = ldexp((double)s->x[d], -32);
    }
}

static void sobol_skip_exact(sobol_t *s, int64_t n)
{
    double x[2 * MAXK + 2];
    for (int64_t i = 0; i < n; ++i) sobol_next(s, x);
}

int qiwo_sobol_points(int D, const uint32_t *m, const uint32_t *x0, int64_t skip, int64_t n,
                      double *out)
{
    sobol_t s;
    sobol_init(&s, D, m, x0);
    sobol_skip_exact(&s, skip);
    for (int64_t i = 0; i < n; ++i) sobol_next(&s, out + i * D);
    return 0;
}

/* Point n (0-based) as UInt32 by the closed form of next!'s recurrence: the shift XOR the
 * columns m[:, b] over the set bits b of the Gray code n ^ (n >> 1).  Pinned against the
 * sequential generator above (and SciPy's) in the tests; used where a sequential skip! to the
 * index would take too long (n near 2^32). */
int qiwo_sobol_point_u32(int D, const uint32_t *m, const uint32_t *x0, uint64_t n, uint32_t *out)
{
    if (n >> 32) return 1;
    const uint64_t g = n ^ (n >> 1);
    for (int d = 0; d < D; ++d) {
        uint32_t v = x0 ? x0[d] : 0u;
        for (int b = 0; b < 32; ++b)
            if ((g >> b) & 1u) v ^= m[d * 32 + b];
        out[d] = v;
    }
    return 0;
}

/* ------------------------------------------------------------------ transforms */

static double simplex_volume(int d, double edge)
{
    /* prod(edge / i for i = 1:d) */
    if (d <= 0) return 1.0;
    double v = 1.0;
    for (int i = 1; i <= d; ++i) v *= edge / (double)i;
    return v;
}

/* src/qmc_integrate.jl:229-238 (RootTransform) */
static void root_map(int d, double u_i, double u_diff, const double *x, double *u)
{
    double w = pow(x[0], 1.0 / d);
    u[0] = w;
    for (int i = 2; i <= d; ++i) {
        w = u[i - 2] * pow(x[i - 1], 1.0 / (double)(d - i + 1));
        u[i - 1] = w;
    }
    for (int i = 0; i < d; ++i) u[i] = u_i + u[i] * u_diff;
}

/* src/qmc_integrate.jl:319-321 (SortTransform): u = u_i .+ sort(x, rev=true) * u_diff */
static void sort_map(int d, double u_i, double u_diff, const double *x, double *u)
{
    for (int i = 0; i < d; ++i) u[i] = x[i];
    for (int i = 1; i < d; ++i)            /* insertion sort, descending */
        for (int j = i; j > 0 && u[j] > u[j - 1]; --j) { double t = u[j]; u[j] = u[j - 1]; u[j - 1] = t; }
    for (int i = 0; i < d; ++i) u[i] = u_i + u[i] * u_diff;
}

/* src/qmc_integrate.jl:138-147 (ExpModelFunctionTransform) */
static void expmodel_map(int d, double u_f, double tau, const double *x, double *u)
{
    u[0] = u_f + tau * log(1 - x[0]);
    for (int i = 1; i < d; ++i) u[i] = u[i - 1] + tau * log(1 - x[i]);
}

/* src/qmc_integrate.jl:425-449 (DoubleSimplexRootTransform) */
static void dsimplex_map(int d_lesser, int d_greater, double u_i, double u_w, double diff_wi,
                         double diff_fw, const double *x, double *u)
{
    int d = d_lesser + d_greater;
    u[0] = pow(x[0], 1.0 / d_greater);
    for (int i = 2; i <= d_greater; ++i)
        u[i - 1] = u[i - 2] * pow(x[i - 1], 1.0 / (double)(d_greater - i + 1));
    for (int i = 0; i < d_greater; ++i) u[i] *= diff_fw;
    for (int i = 0; i < d_greater; ++i) u[i] += u_w;
    if (d_lesser == 0) return;
    u[d_greater] = pow(x[d_greater], 1.0 / d_lesser);
    for (int i = d_greater + 2; i <= d; ++i)
        u[i - 1] = u[i - 2] * pow(x[i - 1], 1.0 / (double)(d - i + 1));
    for (int i = d_greater; i < d; ++i) u[i] *= diff_wi;
    for (int i = d_greater; i < d; ++i) u[i] += u_i;
}

/* ------------------------------------------------------------------ interpolation */

static cplx prop_eval(const qiwo_scalar_gf *g, double dtau)
{
    const cplx *y = (const cplx *)g->data;
    int n = g->n_tau;
    double h = g->h;
    double x = dtau / h;
    int i = (int)floor(x);
    if (i > n - 2) i = n - 2;
    if (i < 0) i = 0;
    double f = x - i;
    if (g->kind == QIWO_INTERP_LINEAR) return y[i] + f * (y[i + 1] - y[i]);
    /* natural cubic spline, second derivatives M (`src/spline_gf.jl:195-202`) */
    const cplx *M = (const cplx *)g->aux;
    double t = f, s = 1.0 - f;
    return s * y[i] + t * y[i + 1] + h * h / 6.0 * ((s * s * s - s) * M[i] + (t * t * t - t) * M[i + 1]);
}

void qiwo_natural_spline_M(int n, double h, const double *y_, double *M_)
{
    const cplx *y = (const cplx *)y_;
    cplx *M = (cplx *)M_;
    for (int i = 0; i < n; ++i) M[i] = 0;
    if (n < 3) return;
    int m = n - 2;
    cplx *dp = malloc(sizeof(cplx) * m);
    double *cp = malloc(sizeof(double) * m);
    for (int i = 0; i < m; ++i) {
        cplx rhs = 6.0 * (y[i + 2] - 2.0 * y[i + 1] + y[i]) / (h * h);
        double den = (i == 0) ? 4.0 : 4.0 - cp[i - 1];
        cp[i] = 1.0 / den;
        dp[i] = (i == 0) ? rhs / den : (rhs - dp[i - 1]) / den;
    }
    M[m] = dp[m - 1];
    for (int i = m - 2; i >= 0; --i) M[i + 1] = dp[i] - cp[i] * M[i + 2];
    free(dp);
    free(cp);
}

/* P block of sector s at dtau >= 0; writes d x d row-major */
static void ppgf_eval(const qiwo_problem *pb, int use_bold, int s, double dtau, cplx *out)
{
    int d = pb->dims[s];
    if (!use_bold) {
        const double *E = pb->atomic_energies + pb->sector_offset[s];
        for (int i = 0; i < d * d; ++i) out[i] = 0;
        /* -i exp(-i dz E) with dz = -i dtau  ==>  -i exp(-dtau E) */
        for (int i = 0; i < d; ++i) out[i * d + i] = -I * exp(-dtau * E[i]);
        return;
    }
    /* linear interpolation of the grid data (kd.interpolate!, topology_eval.jl:368) */
    const qiwo_ppgf *P = &pb->P[s];
    const cplx *data = (const cplx *)P->data; /* [n_tau][d][d] row-major */
    int n = P->n_tau;
    double x = dtau / pb->h;
    int i = (int)floor(x);
    if (i > n - 2) i = n - 2;
    if (i < 0) i = 0;
    double f = x - i;
    const cplx *a = data + (size_t)i * d * d, *b = a + d * d;
    for (int e = 0; e < d * d; ++e) out[e] = a[e] + f * (b[e] - a[e]);
}

/* ------------------------------------------------------------------ evaluator */

enum { NK_PAIR = 1, NK_IDENTITY = 2, NK_INCH = 3, NK_OPERATOR = 4 };

typedef struct {
    int kind, arc, opidx; /* opidx: 1 = head (operator_i), 2 = tail (operator_f) */
} node_t;

typedef struct {
    const qiwo_problem *pb;
    const qiwo_group *gr;
    int n;
    node_t conf[MAXN];
    double times[MAXN];
    int top_to_conf[MAXN];
    int var_pos[MAXN];
    int n_var;                  /* integrated times: 2k minus the fixed pair vertices */
    /* ppgf_mats[i][s]: i*P(t_{i+1}, t_i) */
    cplx *pm;           /* [(n-1)][S] blocks of MAXD*MAXD */
    /* finite-time node matrices: [pos][opslot][s] blocks; op slots: 2*n_pairs (+1 fixed) */
    cplx *nm;
    int nm_nops;
    cplx pair_ints[MAXK][MAXP];
    int sel[MAXK];
    cplx *top_res;      /* [S] blocks */
    cplx *result;       /* [S] blocks */
    /* lazy matrix products, one per final sector */
    const cplx *lmp_mats[MAXS][2 * MAXN];
    int lmp_rows[MAXS][2 * MAXN], lmp_cols[MAXS][2 * MAXN];
    cplx *lmp_prod;     /* [S][2*MAXN] blocks */
    int lmp_nm[MAXS], lmp_np[MAXS];
} evalctx;

#define BLK (MAXD * MAXD)

static cplx *PM(evalctx *e, int i, int s) { return e->pm + ((size_t)i * e->pb->n_sectors + s) * BLK; }
static cplx *NM(evalctx *e, int pos, int op, int s)
{
    return e->nm + (((size_t)pos * e->nm_nops + op) * e->pb->n_sectors + s) * BLK;
}

/* operator block lookup: returns target sector or -1, sets *mat (row-major d_f x d_i) */
static int op_block(const qiwo_problem *pb, int op, int s, const cplx **mat)
{
    int t = pb->op_target[op * pb->n_sectors + s];
    if (t < 0) return -1;
    *mat = (const cplx *)(pb->op_values + 2 * (size_t)pb->op_offset[op * pb->n_sectors + s]);
    return t;
}

static void matmul(int r, int k, int c, const cplx *A, const cplx *B, cplx *C)
{
    for (int i = 0; i < r; ++i)
        for (int j = 0; j < c; ++j) {
            cplx acc = 0;
            for (int l = 0; l < k; ++l) acc += A[i * k + l] * B[l * c + j];
            C[i * c + j] = acc;
        }
}

/* op index inside the node-matrix table for a node at `pos` */
static int node_op_slot_pair(int p, int which) { return 2 * p + (which - 1); }

static void lmp_push(evalctx *e, int sf, const cplx *A, int rows, int cols)
{
    int k = e->lmp_nm[sf]++;
    e->lmp_mats[sf][k] = A;
    e->lmp_rows[sf][k] = rows;
    e->lmp_cols[sf][k] = cols;
}

static void lmp_pop(evalctx *e, int sf)
{
    e->lmp_nm[sf] -= 1;
    if (e->lmp_np[sf] > e->lmp_nm[sf]) e->lmp_np[sf] = e->lmp_nm[sf];
}

/* eval!: partial_prods[n] = A_n * partial_prods[n-1]; result rows(A_N) x cols(A_1) */
static const cplx *lmp_eval(evalctx *e, int sf, int *rows, int *cols)
{
    cplx *pp = e->lmp_prod + (size_t)sf * 2 * MAXN * BLK;
    int c0 = e->lmp_cols[sf][0];
    if (e->lmp_np[sf] == 0) {
        memcpy(pp, e->lmp_mats[sf][0], sizeof(cplx) * e->lmp_rows[sf][0] * c0);
        e->lmp_np[sf] = 1;
    }
    for (int n = e->lmp_np[sf]; n < e->lmp_nm[sf]; ++n)
        matmul(e->lmp_rows[sf][n], e->lmp_cols[sf][n], c0, e->lmp_mats[sf][n],
               pp + (size_t)(n - 1) * BLK, pp + (size_t)n * BLK);
    e->lmp_np[sf] = e->lmp_nm[sf];
    *rows = e->lmp_rows[sf][e->lmp_nm[sf] - 1];
    *cols = c0;
    return pp + (size_t)(e->lmp_nm[sf] - 1) * BLK;
}

static int traverse(evalctx *e, int pos, int s_i, int s_f, cplx w)
{
    const qiwo_problem *pb = e->pb;
    if (pos >= e->n) {
        if (s_i != s_f) return QIWO_ERR_OFFDIAG;
        int r, c;
        const cplx *M = lmp_eval(e, s_f, &r, &c);
        cplx *T = e->top_res + (size_t)s_i * BLK;
        for (int i = 0; i < r * c; ++i) T[i] += w * M[i];
        return 0;
    }
    node_t nd = e->conf[pos];
    int d_i = pb->dims[s_i];
    int rc = 0;
    if (nd.kind == NK_PAIR) {
        if (nd.opidx == 1) {
            for (int p = 0; p < pb->n_pairs; ++p) {
                const cplx *m0;
                int sn = op_block(pb, pb->pair_op_i[p], s_i, &m0);
                if (sn < 0) continue; /* subspace_attachable_pairs[s_i] */
                e->sel[nd.arc] = p;
                lmp_push(e, s_f, NM(e, pos, node_op_slot_pair(p, 1), s_i), pb->dims[sn], d_i);
                rc = traverse(e, pos + 1, sn, s_f, w);
                lmp_pop(e, s_f);
                if (rc) return rc;
            }
        } else {
            int p = e->sel[nd.arc];
            const cplx *m0;
            int sn = op_block(pb, pb->pair_op_f[p], s_i, &m0);
            if (sn >= 0) {
                lmp_push(e, s_f, NM(e, pos, node_op_slot_pair(p, 2), s_i), pb->dims[sn], d_i);
                rc = traverse(e, pos + 1, sn, s_f, e->pair_ints[nd.arc][p] * w);
                lmp_pop(e, s_f);
            }
        }
    } else if (nd.kind == NK_OPERATOR) {
        const cplx *m0;
        int sn = op_block(pb, nd.opidx, s_i, &m0);
        if (sn >= 0) {
            lmp_push(e, s_f, NM(e, pos, 0, s_i), pb->dims[sn], d_i);
            rc = traverse(e, pos + 1, sn, s_f, w);
            lmp_pop(e, s_f);
        }
    } else { /* identity / inch */
        if (pos != 0) lmp_push(e, s_f, NM(e, pos, 0, s_i), d_i, d_i);
        rc = traverse(e, pos + 1, s_i, s_f, w);
        if (pos != 0) lmp_pop(e, s_f);
    }
    return rc;
}

/* Integrated times of a group: 2k minus the fixed pair vertices (PairNode, used by the
   self-energy diagrams of diff_inchworm!, src/inchworm.jl:560-566). */
static int group_D(const qiwo_group *gr)
{
    int D = 2 * gr->order;
    for (int f = 0; f < gr->n_fixed; ++f) D -= gr->fixed_kind[f] == NK_PAIR;
    return D;
}

/* Builds the conf skeleton (fixed nodes) and position maps (topology_eval.jl:254-275). */
static int setup(evalctx *e, const qiwo_problem *pb, const qiwo_group *gr)
{
    memset(e, 0, sizeof(*e));
    e->pb = pb;
    e->gr = gr;
    int n_fixed_nonpair = 0;
    for (int f = 0; f < gr->n_fixed; ++f)
        if (gr->fixed_kind[f] != NK_PAIR) ++n_fixed_nonpair;
    e->n = 2 * gr->order + n_fixed_nonpair;
    if (e->n > MAXN || gr->order > MAXK || pb->n_sectors > MAXS || pb->n_pairs > MAXP) return QIWO_ERR_ARG;
    for (int s = 0; s < pb->n_sectors; ++s)
        if (pb->dims[s] > MAXD) return QIWO_ERR_ARG;
    int is_fixed[MAXN] = {0};
    for (int f = 0; f < gr->n_fixed; ++f) {
        int pos = gr->fixed_pos[f];
        is_fixed[pos] = gr->fixed_kind[f] != NK_PAIR ? 2 : 1;
        e->conf[pos].kind = gr->fixed_kind[f];
        e->conf[pos].opidx = gr->fixed_op[f];
    }
    int k = 0, v = 0;
    for (int pos = e->n - 1; pos >= 0; --pos) {
        if (is_fixed[pos] != 2) e->top_to_conf[k++] = pos;
        if (!is_fixed[pos]) e->var_pos[v++] = pos;
    }
    e->n_var = v;
    int S = pb->n_sectors;
    e->nm_nops = 2 * pb->n_pairs;
    e->pm = calloc((size_t)(e->n > 1 ? e->n - 1 : 1) * S * BLK, sizeof(cplx));
    e->nm = calloc((size_t)e->n * e->nm_nops * S * BLK, sizeof(cplx));
    e->top_res = calloc((size_t)S * BLK, sizeof(cplx));
    e->result = calloc((size_t)S * BLK, sizeof(cplx));
    e->lmp_prod = calloc((size_t)S * 2 * MAXN * BLK, sizeof(cplx));
    if (!e->pm || !e->nm || !e->top_res || !e->result || !e->lmp_prod) return QIWO_ERR_ARG;
    return 0;
}

static void teardown(evalctx *e)
{
    free(e->pm);
    free(e->nm);
    free(e->top_res);
    free(e->result);
    free(e->lmp_prod);
}

/* (eval::TopologyEvaluator)(topologies, times) -- result into e->result */
static int evaluate(evalctx *e, const double *var_times)
{
    const qiwo_problem *pb = e->pb;
    const qiwo_group *gr = e->gr;
    int S = pb->n_sectors, n = e->n;
    for (int f = 0; f < gr->n_fixed; ++f) e->times[gr->fixed_pos[f]] = gr->fixed_time[f];
    for (int j = 0; j < e->n_var; ++j) e->times[e->var_pos[j]] = var_times[j];

    for (int i = 0; i < n - 1; ++i) {
        double ti = e->times[i], tf = e->times[i + 1];
        if (tf < ti) tf = ti;
        for (int s = 0; s < S; ++s) {
            cplx *m = PM(e, i, s);
            int d = pb->dims[s];
            ppgf_eval(pb, gr->use_bold, s, tf - ti, m);
            for (int q = 0; q < d * d; ++q) m[q] *= I;
        }
    }
    /* node matrices: finite-time = mat0 * ppgf(pos-1) (topology_eval.jl:376-388);
       position 0 keeps mat0 */
    for (int pos = 0; pos < n; ++pos) {
        int is_pair = 1, fop = -1;
        for (int f = 0; f < gr->n_fixed; ++f)
            if (gr->fixed_pos[f] == pos && gr->fixed_kind[f] != NK_PAIR) {
                is_pair = 0;
                fop = gr->fixed_kind[f] == NK_OPERATOR ? gr->fixed_op[f] : pb->identity_op;
            }
        int nops = is_pair ? 2 * pb->n_pairs : 1;
        for (int o = 0; o < nops; ++o) {
            int op = is_pair ? (o % 2 == 0 ? pb->pair_op_i[o / 2] : pb->pair_op_f[o / 2]) : fop;
            for (int s = 0; s < S; ++s) {
                const cplx *m0;
                int t = op_block(pb, op, s, &m0);
                if (t < 0) continue;
                int df = pb->dims[t], di = pb->dims[s];
                cplx *dst = NM(e, pos, o, s);
                if (pos == 0) memcpy(dst, m0, sizeof(cplx) * df * di);
                else matmul(df, di, di, m0, PM(e, pos - 1, s), dst);
            }
        }
    }

    for (int s = 0; s < S; ++s) memset(e->result + (size_t)s * BLK, 0, sizeof(cplx) * BLK);

    for (int t = 0; t < gr->n_top; ++t) {
        const int32_t *tp = gr->top_pairs + (size_t)t * 2 * gr->order;
        for (int a = 0; a < gr->order; ++a) {
            int pos_head = e->top_to_conf[tp[2 * a + 1] - 1];
            int pos_tail = e->top_to_conf[tp[2 * a] - 1];
            if (!(pos_tail > pos_head)) return QIWO_ERR_ARG;
            e->conf[pos_head] = (node_t){NK_PAIR, a, 1};
            e->conf[pos_tail] = (node_t){NK_PAIR, a, 2};
            double ti = e->times[pos_head], tf = e->times[pos_tail];
            if (tf < ti) tf = ti;
            for (int p = 0; p < pb->n_pairs; ++p)
                e->pair_ints[a][p] = I * prop_eval(&pb->props[pb->pair_prop[p]], tf - ti);
        }
        for (int s = 0; s < S; ++s) memset(e->top_res + (size_t)s * BLK, 0, sizeof(cplx) * BLK);
        for (int s = 0; s < S; ++s) {
            e->lmp_nm[s] = 0;
            e->lmp_np[s] = 0;
        }
        for (int s_i = 0; s_i < S; ++s_i) {
            int rc = traverse(e, 0, s_i, s_i, 1.0);
            if (rc) return rc;
        }
        cplx coef = -I * (double)gr->top_parity[t] * ((gr->order % 2) ? -1.0 : 1.0);
        for (int s = 0; s < S; ++s) {
            int d = pb->dims[s];
            for (int q = 0; q < d * d; ++q) e->result[(size_t)s * BLK + q] += coef * e->top_res[(size_t)s * BLK + q];
        }
    }
    return 0;
}

typedef struct {
    const qiwo_problem *pb;
    const qiwo_group *gr;
    const uint32_t *m, *x0;
    int64_t first, count, N;
    cplx *out;   /* [S] blocks */
    int rc;
} job_t;

static void *run_range(void *arg)
{
    job_t *jb = arg;
    const qiwo_group *gr = jb->gr;
    const qiwo_problem *pb = jb->pb;
    int S = pb->n_sectors;
    evalctx e;
    jb->rc = setup(&e, pb, gr);
    if (jb->rc) { teardown(&e); return NULL; }
    int D = group_D(gr);
    for (int s = 0; s < S; ++s) memset(jb->out + (size_t)s * BLK, 0, sizeof(cplx) * BLK);

    if (D == 0) {   /* nothing to integrate: one exact evaluation (order 0, order-1 self-energy) */
        jb->rc = evaluate(&e, NULL);
        if (!jb->rc)
            for (int s = 0; s < S; ++s) memcpy(jb->out + (size_t)s * BLK, e.result + (size_t)s * BLK, sizeof(cplx) * BLK);
        teardown(&e);
        return NULL;
    }

    double J;
    if (gr->transform == QIWO_ROOT || gr->transform == QIWO_SORT) J = simplex_volume(D, gr->t_f - gr->t_i);
    else if (gr->transform == QIWO_EXPMODEL) J = 0.0;   /* per sample, below */
    else J = simplex_volume(gr->d_before, gr->t_w - gr->t_i) * simplex_volume(gr->d_after, gr->t_f - gr->t_w);
    /* src/qmc_integrate.jl:158-164: tau^d / exp(-(u_f - u_d) / tau) */
    const double exp_norm = gr->transform == QIWO_EXPMODEL ? pow(gr->decay, (double)D) : 0.0;
    /* prod(branch_direction) over 2k imaginary-branch points: (-i)^(2k) */
    cplx bdir = 1.0;
    for (int j = 0; j < D; ++j) bdir *= -I;

    sobol_t sq;
    sobol_init(&sq, D, jb->m, jb->x0);
    sobol_skip_exact(&sq, jb->first);
    double x[2 * MAXK + 2], u[2 * MAXK + 2];
    for (int64_t i = 0; i < jb->count; ++i) {
        sobol_next(&sq, x);
        if (gr->transform == QIWO_ROOT) root_map(D, gr->t_i, gr->t_f - gr->t_i, x, u);
        else if (gr->transform == QIWO_SORT) sort_map(D, gr->t_i, gr->t_f - gr->t_i, x, u);
        else if (gr->transform == QIWO_EXPMODEL) expmodel_map(D, gr->t_f, gr->decay, x, u);
        else dsimplex_map(gr->d_before, gr->d_after, gr->t_i, gr->t_w, gr->t_w - gr->t_i, gr->t_f - gr->t_w, x, u);
        int neg = 0;
        for (int j = 0; j < D; ++j) if (u[j] < 0.0) neg = 1;
        if (neg) continue;
        if (gr->transform == QIWO_EXPMODEL) J = exp_norm / exp(-(gr->t_f - u[D - 1]) / gr->decay);
        jb->rc = evaluate(&e, u);
        if (jb->rc) break;
        for (int s = 0; s < S; ++s) {
            int d = pb->dims[s];
            for (int q = 0; q < d * d; ++q)
                jb->out[(size_t)s * BLK + q] += (bdir * e.result[(size_t)s * BLK + q]) * J;
        }
    }
    /* rank_weight * (1/N_rank) * res */
    double rank_weight = (double)jb->count / (double)jb->N;
    for (int s = 0; s < S; ++s) {
        int d = pb->dims[s];
        for (int q = 0; q < d * d; ++q)
            jb->out[(size_t)s * BLK + q] = rank_weight * ((1.0 / (double)jb->count) * jb->out[(size_t)s * BLK + q]);
    }
    teardown(&e);
    return NULL;
}

int qiwo_integrate(const qiwo_problem *pb, const qiwo_group *gr, const uint32_t *m,
                   const uint32_t *x0, int64_t N, int n_ranks, double *out)
{
    int S = pb->n_sectors;
    if (n_ranks < 1) n_ranks = 1;
    const int exact = group_D(gr) == 0;
    if (exact) n_ranks = 1;
    job_t *jobs = calloc(n_ranks, sizeof(job_t));
    pthread_t *th = calloc(n_ranks, sizeof(pthread_t));
    cplx *bufs = calloc((size_t)n_ranks * S * BLK, sizeof(cplx));
    int64_t q = exact ? 1 : N / n_ranks, r = exact ? 0 : N % n_ranks, start = 0;
    for (int k = 0; k < n_ranks; ++k) {
        int64_t cnt = q + (k < r ? 1 : 0);
        jobs[k] = (job_t){pb, gr, m, x0, start, cnt, N, bufs + (size_t)k * S * BLK, 0};
        start += cnt;
    }
    for (int k = 1; k < n_ranks; ++k)
        if (jobs[k].count > 0) pthread_create(&th[k], NULL, run_range, &jobs[k]);
    if (jobs[0].count > 0) run_range(&jobs[0]);
    int rc = jobs[0].rc;
    for (int k = 1; k < n_ranks; ++k) {
        if (jobs[k].count > 0) pthread_join(th[k], NULL);
        if (jobs[k].rc) rc = jobs[k].rc;
    }
    /* all_reduce!(res, +) in rank order; output: per sector s the d_s x d_s block row-major */
    size_t off = 0;
    for (int s = 0; s < S; ++s) {
        int d = pb->dims[s];
        for (int e = 0; e < d * d; ++e) {
            cplx acc = 0;
            for (int k = 0; k < n_ranks; ++k)
                if (jobs[k].count > 0) acc += jobs[k].out[(size_t)s * BLK + e];
            out[2 * (off + e)] = creal(acc);
            out[2 * (off + e) + 1] = cimag(acc);
        }
        off += (size_t)d * d;
    }
    free(jobs);
    free(th);
    free(bufs);
    return rc;
}

/* One rank's share: samples [first, first + count) of N_total, weighted count/N_total
 * (rank_weight * contour_integral over the rank's range, src/inchworm.jl:168-187). */
int qiwo_integrate_range(const qiwo_problem *pb, const qiwo_group *gr, const uint32_t *m, const uint32_t *x0,
                         int64_t first, int64_t count, int64_t N_total, double *out)
{
    int S = pb->n_sectors;
    cplx *buf = calloc((size_t)S * BLK, sizeof(cplx));
    const int exact = group_D(gr) == 0;
    job_t jb = (job_t){pb, gr, m, x0, first, exact ? 1 : count, exact ? 1 : N_total, buf, 0};
    if (jb.count > 0) run_range(&jb);
    size_t off = 0;
    for (int s = 0; s < S; ++s) {
        int d = pb->dims[s];
        for (int e = 0; e < d * d; ++e) {
            cplx v = jb.count > 0 ? buf[(size_t)s * BLK + e] : 0;
            out[2 * (off + e)] = creal(v);
            out[2 * (off + e) + 1] = cimag(v);
        }
        off += (size_t)d * d;
    }
    free(buf);
    return jb.rc;
}
