// mdg_nonbonded_quarter.cu -- the pair kernel with 8-atom i groups per
// quarter warp (launch-shape option), instantiated apart from the other
// forms so they compile in parallel.
#include "mdg_nonbonded_kernel.cuh"

namespace mdg {
namespace {

template <int COUL, bool LJ, bool SW>
cudaError_t dispatch_nb_q(mdg_system *s, const NbArgs &a, int energy, int dump) {
    dim3 grid(a.persistent ? s->nb_persistent_ctas : a.n_items), block(32);
    if (a.persistent && cudaMemsetAsync(a.queue, 0, sizeof(int), s->stream) != cudaSuccess)
        return cudaGetLastError();
    if (dump) {
        if constexpr (COUL == MDG_COUL_EWALD && LJ && !SW)
            k_nonbonded_q<COUL, LJ, SW, false, true><<<grid, block, 0, s->stream>>>(a);
    } else if (energy)
        k_nonbonded_q<COUL, LJ, SW, true, false><<<grid, block, 0, s->stream>>>(a);
    else
        k_nonbonded_q<COUL, LJ, SW, false, false><<<grid, block, 0, s->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t dispatch_shape_q(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj, bool sw,
                             int energy, int dump) {
    if (dump) return dispatch_nb_q<MDG_COUL_EWALD, true, false>(s, a, 0, 1);
    if (coul_tile == MDG_COUL_EWALD && !want_lj)
        return dispatch_nb_q<MDG_COUL_EWALD, false, false>(s, a, energy, dump);
    if (coul_tile == MDG_COUL_EWALD)
        return sw ? dispatch_nb_q<MDG_COUL_EWALD, true, true>(s, a, energy, dump)
                  : dispatch_nb_q<MDG_COUL_EWALD, true, false>(s, a, energy, dump);
    return sw ? dispatch_nb_q<MDG_COUL_NONE, true, true>(s, a, energy, dump)
              : dispatch_nb_q<MDG_COUL_NONE, true, false>(s, a, energy, dump);
}

}  // namespace

cudaError_t launch_nb_quarter(mdg_system *s, const NbArgs &a, int coul_tile, bool want_lj,
                              bool sw, int energy, int dump) {
    return dispatch_shape_q(s, a, coul_tile, want_lj, sw, energy, dump);
}

}  // namespace mdg
