// mdg_nonbonded_half.cu -- the pair kernel with 16-atom i groups per half
// warp (launch-shape option), instantiated apart from the whole-warp kernel
// so the two compile in parallel.
#include "mdg_nonbonded_kernel.cuh"

namespace mdg {

cudaError_t launch_nb_half(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj, bool sw,
                           int energy, int dump) {
    return dispatch_shape<true>(s, a, coul_tile, want_lj, sw, energy, dump);
}

}  // namespace mdg
