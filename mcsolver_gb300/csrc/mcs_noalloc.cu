// mcs_noalloc.cu -- allocation-free Ising sweeps for callers that cannot call cudaMalloc.
//
// Some callers own all device memory themselves: a host framework with its
// own caching allocator, a process that has reserved the GPU's memory up front,
// or code running where a cudaMalloc would stall or fail (inside another
// library's allocation scope).  mcs_ising_square_noalloc() runs Metropolis
// sweeps of a 2D square-lattice Ising model on a spin array the caller holds in
// device memory and writes per-sweep sums to a device array the caller holds;
// the library allocates nothing, neither device nor pinned memory.
//
// The sweep is the engine's own: the same colour order, the same Philox words
// (colour-local index k, sweep t, colour c), the same integer acceptance
// thresholds ceil(exp(corr) * 2^32) as the Ising path of mcs_solve(), so the
// spins after n sweeps are the ones mcs_solve() produces for the same lattice,
// couplings and seed.  The only scratch it needs -- per-block partial sums of
// the reduction and the completion counter of the last-block pattern -- lives
// in the file-scope array g_noalloc_scratch below, of fixed size, held by every
// GPU that loads this library until the process exits.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/mcsgpu.h"
#include "mcs_device.cuh"
#include "mcs_engine.h"

namespace mcs {

#define NA_THREADS 256
#define NA_SITES_PER_BLOCK (4 * NA_THREADS)  // four sites per thread and colour
#define NA_MAX_BLOCKS 4096                   // blocks of the reduction kernel
#define NA_MAX_SITES (2LL * NA_MAX_BLOCKS * NA_SITES_PER_BLOCK)

// [NA_MAX_BLOCKS][2] partial sums, then one completion counter.
// 4096*2*8 + 256 bytes = 64.25 KiB per device.
static __device__ __align__(256) long long g_noalloc_scratch[2 * NA_MAX_BLOCKS + 32];

struct NaThr {
    unsigned long long t[2][5];  // [sigma_i > 0][number of + neighbours]
};

// one colour of one sweep, sites in the caller's order i = x*Ly + y
__global__ void __launch_bounds__(NA_THREADS) k_na_colour(signed char *s, int Lx, int Ly, NaThr thr,
                                                           unsigned long long seed, long long t, int c)
{
    const int hy = Ly >> 1, nc = (Lx * Ly) >> 1;
    const int q = blockIdx.x * NA_THREADS + threadIdx.x;
    const int k0 = 4 * q;
    if (k0 >= nc) return;
    const uint4 w = philox_t((uint32_t)q, t, (uint32_t)c, seed);
    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int k = k0 + e;
        if (k >= nc) break;
        const int x = k / hy, yh = k - x * hy;
        const int y = 2 * yh + ((x + c) & 1);
        const int xp = x + 1 == Lx ? 0 : x + 1, xm = x == 0 ? Lx - 1 : x - 1;
        const int yp = y + 1 == Ly ? 0 : y + 1, ym = y == 0 ? Ly - 1 : y - 1;
        const int i = x * Ly + y;
        const int np = (s[xp * Ly + y] > 0) + (s[xm * Ly + y] > 0) + (s[x * Ly + yp] > 0) + (s[x * Ly + ym] > 0);
        const int si = s[i];
        if ((unsigned long long)ws[e] < thr.t[si > 0][np]) s[i] = (signed char)(-si);
    }
}

// sum of sigma and of sigma_i*sigma_j over the bonds (each bond once); the
// last block to finish adds the partials (all its threads, then a block sum:
// the sums are integers, so the order does not change them) and writes
// out[0..1]
__global__ void __launch_bounds__(NA_THREADS) k_na_sums(const signed char *s, int Lx, int Ly, long long *scratch,
                                                         long long *out)
{
    __shared__ long long red[32 * 2 + 2];
    __shared__ bool last;
    const int N = Lx * Ly;
    long long a[2] = {0, 0};
    for (int i = blockIdx.x * NA_THREADS + threadIdx.x; i < N; i += gridDim.x * NA_THREADS) {
        const int x = i / Ly, y = i - x * Ly;
        const int xp = x + 1 == Lx ? 0 : x + 1, yp = y + 1 == Ly ? 0 : y + 1;
        const int si = s[i];
        a[0] += si;
        a[1] += si * (s[xp * Ly + y] + s[x * Ly + yp]);
    }
    block_sum_ll<2>(a, red, red + 64);
    unsigned int *counter = (unsigned int *)(scratch + 2 * NA_MAX_BLOCKS);
    if (threadIdx.x == 0) {
        scratch[2 * blockIdx.x] = red[64];
        scratch[2 * blockIdx.x + 1] = red[65];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {  // the same for every thread of the block
        __threadfence();
        long long p[2] = {0, 0};
        for (unsigned g = threadIdx.x; g < gridDim.x; g += NA_THREADS) {
            p[0] += ((volatile long long *)scratch)[2 * g];
            p[1] += ((volatile long long *)scratch)[2 * g + 1];
        }
        block_sum_ll<2>(p, red, red + 64);
        if (threadIdx.x == 0) {
            out[0] = red[64];
            out[1] = red[65];
            *counter = 0u;  // ready for the next sweep
        }
    }
}

// Device address of the scratch array on the current device, looked up on
// every call (cheap once the module is loaded, and never stale after a
// cudaDeviceReset).  The first call on a device also loads both kernels
// (under lazy module loading a kernel is otherwise loaded at its first launch,
// which may allocate device memory for the module, even inside a capture).
static std::mutex g_na_mutex;
static bool g_na_loaded[64];

static int noalloc_scratch(cudaStream_t st, long long **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)); return MCS_ECUDA; }
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return MCS_EINVAL; }
    if (st) {
        int sdev = -1;
        e = cudaStreamGetDevice(st, &sdev);
        if (e != cudaSuccess) { set_error(std::string("cudaStreamGetDevice: ") + cudaGetErrorString(e)); return MCS_EINVAL; }
        if (sdev != dev) {
            set_error("the stream belongs to device " + std::to_string(sdev) + " but device " + std::to_string(dev) +
                      " is current");
            return MCS_EINVAL;
        }
    }
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_loaded[dev]) {
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, k_na_colour);
            if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_na_sums);
            if (e != cudaSuccess) { set_error(std::string("loading the kernels: ") + cudaGetErrorString(e)); return MCS_ECUDA; }
            g_na_loaded[dev] = true;
        }
    }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        return MCS_ECUDA;
    }
    *out = (long long *)p;
    return MCS_OK;
}

}  // namespace mcs

using namespace mcs;

extern "C" int mcs_ising_square_noalloc(int8_t *d_sigma, int32_t Lx, int32_t Ly, double K, double h, uint64_t seed,
                                        int64_t sweep0, int32_t nsweeps, int64_t *d_sums, void *stream)
{
    if (!d_sigma || !d_sums) { set_error("null device pointer"); return MCS_EINVAL; }
    if (Lx < 4 || Ly < 4 || (Lx & 1) || (Ly & 1)) { set_error("Lx and Ly must be even and >= 4"); return MCS_EINVAL; }
    if ((long long)Lx * Ly > NA_MAX_SITES) {
        set_error("lattice larger than the fixed scratch allows (" + std::to_string(NA_MAX_SITES) + " sites)");
        return MCS_EINVAL;
    }
    if (nsweeps < 0 || sweep0 < 0) { set_error("negative sweep count or index"); return MCS_EINVAL; }
    cudaStream_t st = (cudaStream_t)stream;
    long long *scratch = nullptr;
    int rc = noalloc_scratch(st, &scratch);
    if (rc != MCS_OK) return rc;
    // acceptance thresholds, evaluated as the Ising table of mcs_solve():
    // corr = 2 (sigma * K * (2 n+ - 4) - h * sigma), threshold ceil(exp(corr) 2^32)
    NaThr thr;
    for (int sg = 0; sg < 2; ++sg)
        for (int np = 0; np <= 4; ++np) {
            const double sigma = sg ? 1.0 : -1.0;
            double sumq = 0.0;
            sumq += K * (2 * np - 4);
            const double corr = 2 * (sigma * sumq - h * 1.0 * sigma);
            unsigned long long t;
            if (corr >= 0) t = 1ULL << 32;
            else {
                const double x = ceil(exp(corr) * 4294967296.0);
                t = x >= 4294967296.0 ? (1ULL << 32) : (unsigned long long)x;
            }
            thr.t[sg][np] = t;
        }
    const int N = Lx * Ly;
    const int nq = (N / 2 + 3) / 4;
    const int gsweep = (nq + NA_THREADS - 1) / NA_THREADS;
    // about 16 sites per thread: fewer partials for the last block to add
    const int gsum = std::min(NA_MAX_BLOCKS, std::max(1, (N + 16 * NA_THREADS - 1) / (16 * NA_THREADS)));
    // the completion counter must start at zero (a previous call may have been interrupted)
    cudaError_t e = cudaMemsetAsync(scratch + 2 * NA_MAX_BLOCKS, 0, sizeof(unsigned int), st);
    for (int k = 0; k < nsweeps && e == cudaSuccess; ++k) {
        const long long t = sweep0 + k;
        for (int c = 0; c < 2 && e == cudaSuccess; ++c) {
            k_na_colour<<<gsweep, NA_THREADS, 0, st>>>((signed char *)d_sigma, Lx, Ly, thr, seed, t, c);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        k_na_sums<<<gsum, NA_THREADS, 0, st>>>((const signed char *)d_sigma, Lx, Ly, scratch, (long long *)d_sums + 2 * k);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) { set_error(std::string("noalloc launch: ") + cudaGetErrorString(e)); return MCS_ECUDA; }
    return MCS_OK;
}
