// k_grid_gcf instantiations for supports 25-31 (odd).
#include "gcf_grid_kernel.cuh"

namespace ngg {
int launch_grid_gcf_hi(const GArgs &a, bool data, unsigned blocks, cudaStream_t s) {
    switch (a.S) {
        case 25: launch_one<25>(a, data, blocks, s); break;
        case 27: launch_one<27>(a, data, blocks, s); break;
        case 29: launch_one<29>(a, data, blocks, s); break;
        case 31: launch_one<31>(a, data, blocks, s); break;
        default: return fail(NGG_ERR_UNSUPPORTED, "support class");
    }
    NGG_CHECK_LAUNCH("k_grid_gcf");
    return NGG_OK;
}
}  // namespace ngg
