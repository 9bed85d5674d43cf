/*
 * nnp.h -- FP64 CPU restatement of the NNP force (test infrastructure only;
 * see nnp.c for the definitions and the n2p2 provenance).
 */
#ifndef GBMD_ORACLE_NNP_H
#define GBMD_ORACLE_NNP_H

#include "oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NNP_MAXSF 64
#define ORC_NNP_MAXLAYERS 4
#define ORC_NNP_MAXNODES 64

/* One element.  Weight layer l (1..nlayers) maps nodes[l-1] -> nodes[l]:
 * W_l[j][i] at w[woff[l] + j * nodes[l-1] + i], bias b[boff[l] + j]. */
typedef struct
{
    int nsf;
    int type[ORC_NNP_MAXSF]; /* 2 radial, 3 angular */
    /* neighbour elements (0-based, atomic-number order): e1 for a radial
     * function; the unordered pair {e1, e2} for an angular one */
    int e1[ORC_NNP_MAXSF], e2[ORC_NNP_MAXSF];
    double eta[ORC_NNP_MAXSF], rs[ORC_NNP_MAXSF], lambda[ORC_NNP_MAXSF],
        zeta[ORC_NNP_MAXSF], rc[ORC_NNP_MAXSF];
    double gmin[ORC_NNP_MAXSF], gmax[ORC_NNP_MAXSF];
    double smin, smax;
    int nlayers;
    int nodes[ORC_NNP_MAXLAYERS + 1];
    char act[ORC_NNP_MAXLAYERS + 1];
    int woff[ORC_NNP_MAXLAYERS + 1], boff[ORC_NNP_MAXLAYERS + 1];
    const double *w, *b;
    double e_offset, conv_energy, mean_energy;
} orc_nnp;

/* Symmetry functions G[n][nsf], energies E[n], dE/dG [n][nsf] and forces
 * f[n][3] (accumulated; caller zeroes) over a full list; any output may be
 * NULL.  Returns sum_i E_i in network units. */
double orc_nnp_compute( int64_t n, const double *x, const orc_list *l, const double L[3],
                        const orc_nnp *m, double *G, double *E, double *dEdG, double *f );
/* Several elements: atom i uses models[type[i]]; G and dEdG rows have
 * gstride entries (>= every element's nsf). */
double orc_nnp_compute_multi( int64_t n, const double *x, const int32_t *type, const orc_list *l,
                              const double L[3], const orc_nnp *models, int nelem, int gstride,
                              double *G, double *E, double *dEdG, double *f );
/* The same on nthreads OpenMP threads (results equal the serial ones up to
 * the order in which the force contributions of different threads add). */
double orc_nnp_compute_multi_mt( int64_t n, const double *x, const int32_t *type,
                                 const orc_list *l, const double L[3], const orc_nnp *models,
                                 int nelem, int gstride, double *G, double *E, double *dEdG,
                                 double *f, int nthreads );
/* CbnMD::init + run with the NNP force (see nnp.c); returns the thermo row
 * count or -1. */
int orc_run_nnp( int64_t n, double *x, double *v, double *f, int32_t *type, int32_t *id,
                 const double lo[3], const double hi[3], const orc_nnp *models, int nelem,
                 orc_run_cfg *cfg, double *thermo, int max_rows, int snap_step, double *snap_x,
                 double *snap_v, double *snap_f, int32_t *snap_id );
/* ForceNNP::compute_energy's assembly of the total. */
double orc_nnp_energy( int64_t n, double esum, const orc_nnp *m );

#ifdef __cplusplus
}
#endif
#endif
