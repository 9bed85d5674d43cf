// gbmd_nnp.cu -- neural-network potential (Behler-Parrinello symmetry
// functions, per-element MLP, forces).  Placeholder until the NNP kernels
// land: every entry point reports that the potential is not available.
#include "gbmd_internal.cuh"

struct NnpModel
{
    int dummy;
};

int gbmd_nnp_launch( gbmd_ctx *c, bool )
{
    return gbmd_fail( c, GBMD_ERR_ARG, "NNP force not available in this build" );
}

void gbmd_nnp_free( gbmd_ctx *c )
{
    delete c->nnp;
    c->nnp = nullptr;
}

extern "C" int gbmd_nnp_load( gbmd_ctx *c, const char *, double, double )
{
    if ( !c )
        return GBMD_ERR_ARG;
    return gbmd_fail( c, GBMD_ERR_ARG, "NNP force not available in this build" );
}

extern "C" int gbmd_nnp_download( gbmd_ctx *c, double *, double *, int * )
{
    if ( !c )
        return GBMD_ERR_ARG;
    return gbmd_fail( c, GBMD_ERR_ARG, "NNP force not available in this build" );
}
