// mdg_noalloc.cu -- per-system kinetic energies through an entry point that
// allocates no device memory.
//
// Who needs it: callers that must not have device memory allocated behind
// their back -- a host program whose own pool already owns the GPU's memory
// (it reserves it up front and hands out every buffer itself, so a library
// cudaMalloc either fails or breaks its accounting), or a tight loop that
// cannot afford cudaMalloc/cudaFree, which may synchronise the whole device
// and stall every other stream.
//
// mdg_kinetic_energies_noalloc computes what mdg_kinetic_energy computes (the
// same kernel arithmetic and the same FP64-block / int64 fixed-point
// reduction), but accumulates into a file-scope static device array instead
// of the system's energy buffer, so the call makes no cudaMalloc/cudaFree and
// calls no allocating library routine.  The array holds kEnergySlots int64
// words per system for at most MDG_NOALLOC_MAX_SYSTEMS systems (128 KiB,
// held by every GPU that loads the library until the process exits); a
// larger batch is rejected.
//
// The array's device address is looked up once per device (the first call
// on that device, with the device current) with cudaGetSymbolAddress; make
// that first call before any stream capture.  All calls share the one
// array and each call zeroes it first: calls that overlap in time (two host
// threads, or two streams whose work overlaps) race on it.
#include <mutex>

#include "mdg_internal.cuh"

namespace mdg {
namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) long long g_scratch[kEnergySlots * MDG_NOALLOC_MAX_SYSTEMS];

std::mutex g_scratch_mutex;
long long *g_scratch_ptr[kMaxDevices] = {};

__global__ void __launch_bounds__(256) k_kinetic_scratch(const double *__restrict__ v,
                                                         const double *__restrict__ mass, int n,
                                                         const int *__restrict__ atom_sys,
                                                         long long *__restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0;
    if (i < n) ke = 0.5 * mass[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                                     v[3 * i + 2] * v[3 * i + 2]);
    const double e[1] = {ke};
    const int slot[1] = {kSlotKinetic};
    block_energy_add<1>(acc, i < n ? atom_sys[i] : -1, e, slot);
}

}  // namespace

// device address of the scratch array on `device` (current); 0 on failure
cudaError_t noalloc_scratch(int device, long long **out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[device] = (long long *)p;
    }
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

cudaError_t launch_kinetic_scratch(mdg_system *s, long long *acc) {
    k_kinetic_scratch<<<(s->n + 255) / 256, 256, 0, s->stream>>>(s->v, s->mass, s->n,
                                                                 s->atom_sys, acc);
    return cudaGetLastError();
}

}  // namespace mdg
