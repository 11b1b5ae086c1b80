/*
 * CPU oracle for the qMC diagram-integration path -- test infrastructure only.
 * Layouts (all 0-based, complex numbers as interleaved (re, im) doubles):
 *   operator block of op o from sector s: values at op_values[2*op_offset[o*S+s] ...],
 *       row-major d_f x d_i, target sector op_target[o*S+s] (-1: no block);
 *   bold P of sector s: data [n_tau][d][d] row-major (P_s(tau_j, 0), carrying -i);
 *   scalar propagators: data [n_tau] (Delta(tau_j), carrying -i).
 */
#ifndef QIW_ORACLE_H
#define QIW_ORACLE_H
#include <stdint.h>

#define QIWO_ERR_ARG 1
#define QIWO_ERR_OFFDIAG 2

enum { QIWO_INTERP_LINEAR = 0, QIWO_INTERP_CUBIC = 1 };
enum { QIWO_ROOT = 0, QIWO_DSIMPLEX = 1, QIWO_SORT = 2, QIWO_EXPMODEL = 3 };

typedef struct {
    int kind;          /* QIWO_INTERP_LINEAR or QIWO_INTERP_CUBIC */
    int n_tau;
    double h;
    const double *data; /* [n_tau] complex */
    const double *aux;  /* cubic: second derivatives M [n_tau] complex */
} qiwo_scalar_gf;

typedef struct {
    int kind;          /* QIWO_INTERP_LINEAR (the only rule the evaluator applies to P) */
    int n_tau;
    int n_valid;       /* informational: number of grid points already computed */
    const double *data; /* [n_tau][d][d] complex */
    const double *der;  /* unused by the evaluator */
} qiwo_ppgf;

typedef struct {
    int n_sectors;
    const int32_t *dims;
    const int32_t *sector_offset;   /* prefix sums of dims */
    double beta, h;
    const double *atomic_energies;  /* E + lambda, [sum d] */
    const qiwo_ppgf *P;             /* [n_sectors] */
    int n_ops;
    const int32_t *op_target;       /* [n_ops * S] */
    const int64_t *op_offset;       /* [n_ops * S] complex-element offsets */
    const double *op_values;
    int identity_op;
    int n_pairs;
    const int32_t *pair_op_i, *pair_op_f, *pair_prop;
    const qiwo_scalar_gf *props;
} qiwo_problem;

typedef struct {
    int order;
    int use_bold;
    int transform;     /* QIWO_ROOT, QIWO_SORT or QIWO_EXPMODEL (bare), QIWO_DSIMPLEX (bold, correlator) */
    int d_before, d_after;
    double t_i, t_w, t_f;
    int n_fixed;
    const int32_t *fixed_pos;    /* 0-based configuration positions */
    const int32_t *fixed_kind;   /* 2 identity, 3 inch, 4 operator */
    const int32_t *fixed_op;     /* operator index for kind 4 */
    const double *fixed_time;
    int n_top;
    const int32_t *top_pairs;    /* [n_top][order][2], 1-based topology vertices */
    const int32_t *top_parity;   /* [n_top] */
    double decay;                /* QIWO_EXPMODEL: decay rate tau of the model function */
} qiwo_group;

int qiwo_sobol_directions(int D, const int64_t *poly, const int64_t *vinit, int vinit_cols, uint32_t *m);
int qiwo_sobol_points(int D, const uint32_t *m, const uint32_t *x0, int64_t skip, int64_t n, double *out);
int qiwo_sobol_point_u32(int D, const uint32_t *m, const uint32_t *x0, uint64_t n, uint32_t *out);
void qiwo_natural_spline_M(int n, double h, const double *y, double *M);
int qiwo_integrate(const qiwo_problem *pb, const qiwo_group *gr, const uint32_t *m, const uint32_t *x0,
                   int64_t N, int n_ranks, double *out);

int qiwo_integrate_range(const qiwo_problem *pb, const qiwo_group *gr, const uint32_t *m, const uint32_t *x0,
                         int64_t first, int64_t count, int64_t N_total, double *out);

#endif
