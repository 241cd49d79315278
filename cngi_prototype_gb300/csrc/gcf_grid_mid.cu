// k_grid_gcf instantiations for supports 17-23 (odd).
#include "gcf_grid_kernel.cuh"

namespace ngg {
int launch_grid_gcf_mid(const GArgs &a, bool data, unsigned blocks, cudaStream_t s) {
    switch (a.S) {
        case 17: launch_one<17>(a, data, blocks, s); break;
        case 19: launch_one<19>(a, data, blocks, s); break;
        case 21: launch_one<21>(a, data, blocks, s); break;
        case 23: launch_one<23>(a, data, blocks, s); break;
        default: return fail(NGG_ERR_UNSUPPORTED, "support class");
    }
    NGG_CHECK_LAUNCH("k_grid_gcf");
    return NGG_OK;
}
}  // namespace ngg
