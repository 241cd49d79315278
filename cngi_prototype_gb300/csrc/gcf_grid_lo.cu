// k_grid_gcf instantiations for supports 1-15 (odd).
#include "gcf_grid_kernel.cuh"

namespace ngg {
int launch_grid_gcf_lo(const GArgs &a, bool data, unsigned blocks, cudaStream_t s) {
    switch (a.S) {
        case 1: launch_one<1>(a, data, blocks, s); break;
        case 3: launch_one<3>(a, data, blocks, s); break;
        case 5: launch_one<5>(a, data, blocks, s); break;
        case 7: launch_one<7>(a, data, blocks, s); break;
        case 9: launch_one<9>(a, data, blocks, s); break;
        case 11: launch_one<11>(a, data, blocks, s); break;
        case 13: launch_one<13>(a, data, blocks, s); break;
        case 15: launch_one<15>(a, data, blocks, s); break;
        default: return fail(NGG_ERR_UNSUPPORTED, "support class");
    }
    NGG_CHECK_LAUNCH("k_grid_gcf");
    return NGG_OK;
}
}  // namespace ngg
