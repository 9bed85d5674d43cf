// gbmd_nnp.cuh -- NNP model structures shared by the symmetry-function /
// force kernels (gbmd_nnp.cu) and the tensor-core MLP (gbmd_nnp_mlp_tc.cu).
#pragma once

#include "gbmd_internal.cuh"

#define NNP_MAXSF 64
#define NNP_MAXNODES 64
#define NNP_MAXLAYERS 4
#define NNP_MAXNBR 192 // neighbours inside rc per atom (flagged if exceeded)
#define NNP_WARPS_F 4 // warps per block, FP32 instantiation
#define NNP_WARPS_D 2 // FP64 (twice the shared memory per warp)
#define NNP_MAXETA 4 // distinct angular eta (grid rows)
#define NNP_MAXLZ 8  // distinct angular (lambda, zeta) (grid columns)

// Device-side model (one element).
struct NnpParams
{
    int nsf, nrad, nang;
    double rc;
    double eta_r[NNP_MAXSF], rs_r[NNP_MAXSF];
    int ang_eta[NNP_MAXSF], ang_lz[NNP_MAXSF];
    int grid_sf[NNP_MAXETA][NNP_MAXLZ]; // angular function of (eta, (lambda, zeta)) or -1
    double ang_pre[NNP_MAXSF]; // 2^(1 - zeta)
    int neta, nlz;
    double eta_u[NNP_MAXETA];
    double lam_u[NNP_MAXLZ];
    double zeta_u[NNP_MAXLZ];
    int zeta_int[NNP_MAXLZ]; // >0: integer power by multiplication
    double gmin[NNP_MAXSF], gscale[NNP_MAXSF];
    double smin;
    int nl;                          // weight layers
    int nodes[NNP_MAXLAYERS + 1];    // nodes[0] = nsf
    char act[NNP_MAXLAYERS + 1];     // act[l] for l >= 1
    int woff[NNP_MAXLAYERS + 1], boff[NNP_MAXLAYERS + 1];
    double e_offset;
    double cflength, cfenergy;
};

struct NnpModel
{
    NnpParams p{};
    std::vector<double> w, b; // host copies
    double *d_w = nullptr, *d_b = nullptr;
    float *d_wf = nullptr, *d_bf = nullptr;
    DevBuf<double> G, dEdG, E; // per atom
    std::string dir;
    struct TcModel *d_tc = nullptr; // tensor-core MLP operands (when the shape fits)
};

// Tensor-core MLP (mixed precision): operand images and FP32 constants.
// Each B image is one 32 (N) x 96 (K) BF16 operand in the no-swizzle
// K-major core-matrix layout: element (n, k) at byte
// ((n / 8) * 12 + k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2.  K holds the
// split-BF16 copies [hi | hi | lo] of the FP32 matrix so that one K = 96
// chain computes hi*hi + lo*hi + hi*lo against an A of [hi | lo | hi].
#define TC_B_BYTES ( 4 * 12 * 128 )
struct TcModel
{
    uint16_t img[4][TC_B_BYTES / 2]; // forward W1, forward W2, backward W2^T, backward W1^T
    float b1[32], b2[32], w3[32], b3;
    float gmin[32], gscale[32], smin;
    int nsf, h1, h2;
    char act1, act2;
};

// Build the tensor-core operands when the network fits (nsf, hidden <= 32,
// two hidden layers, linear output); returns false otherwise.
bool gbmd_tc_model_build( const NnpParams &p, const std::vector<double> &w,
                          const std::vector<double> &b, TcModel &out );
int gbmd_nnp_mlp_tc_launch( gbmd_ctx *c, const TcModel *dev, const float *G, float *dEdG,
                            double *E, int n, double *partials ); // gbmd_nnp_mlp_tc.cu

