// nb_bh.cu -- Barnes-Hut pipeline (placeholder until the octree kernels land).
#include "nb_internal.h"

namespace nb {
struct BHTree {
    int dummy = 0;
};
BHTree *bh_create() { return new BHTree(); }
void bh_destroy(BHTree *t) { delete t; }
nb_status bh_compute(BHTree *, const double *, const double *, const double *, const double *,
                     int, double, double, double, int, double *, double *, double *,
                     cudaStream_t, const KernelTimer *)
{
    return fail(NB_ERR_UNSUPPORTED, "Barnes-Hut not built yet");
}
nb_status bh_info(BHTree *, cudaStream_t, nb_bh_info *) { return fail(NB_ERR_UNSUPPORTED, "bh"); }
nb_status bh_read_order(BHTree *, cudaStream_t, uint64_t *, uint32_t *)
{
    return fail(NB_ERR_UNSUPPORTED, "bh");
}
nb_status bh_read_nodes(BHTree *, cudaStream_t, int, int *, uint64_t *, int *, int *, int *,
                        int *, int *, float *)
{
    return fail(NB_ERR_UNSUPPORTED, "bh");
}
} // namespace nb
