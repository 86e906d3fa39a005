// mcs_pt.cu -- parallel-tempering exchange step on the device.
//
// Replicas hold configurations; temperature slots hold the inverse
// temperature and the observable accumulators of that temperature.  After
// every sweep neighbouring slots (k, k+1) with k of the sweep's parity try to
// exchange their configurations with probability
//     min(1, exp((beta_k - beta_{k+1}) (E_k - E_{k+1})))
// (E in the problem's physical units).  An exchange swaps the
// temperature-attached fields of the two replica descriptors -- beta and the
// accumulator array -- and swaps the configuration energies back, so each
// configuration keeps its spins, energy and Philox key.  The reference has no
// exchange step (it runs each temperature on its own, win.py:440-444).
#include <cuda_runtime.h>

#include "mcs_device.cuh"
#include "mcs_internal.h"

namespace mcs {

__global__ void k_pt_exchange(Rep *reps, int nt, int *perm, unsigned long long seed, long long *acc_cnt,
                              long long *att_cnt)
{
    // one thread per candidate pair; pairs of one parity are disjoint
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const Rep &R0 = reps[perm[0]];
    const long long t = R0.u;  // sweeps done so far (all replicas move in lockstep)
    if (R0.u > R0.units_total || t == 0) return;
    const int parity = (int)((t - 1) & 1);
    const int k = 2 * tid + parity;
    if (k + 1 >= nt) return;
    Rep &A = reps[perm[k]];
    Rep &B = reps[perm[k + 1]];
    const double ea = A.acc[A_ECUR], eb = B.acc[A_ECUR];
    const double arg = ((double)A.beta - (double)B.beta) * (ea - eb);
    const uint4 w = philox((uint32_t)k, (uint32_t)t, (uint32_t)((unsigned long long)t >> 32), 0x6000u, seed);
    const bool acc = arg >= 0.0 || exp(arg) > (double)w.x * (1.0 / 4294967296.0);
    atomicAdd((unsigned long long *)&att_cnt[k], 1ULL);
    if (!acc) return;
    atomicAdd((unsigned long long *)&acc_cnt[k], 1ULL);
    // temperature-attached fields change hands ...
    const float bA = A.beta;
    A.beta = B.beta; B.beta = bA;
    double *aA = A.acc;
    A.acc = B.acc; B.acc = aA;
    double *sA = A.series;
    A.series = B.series; B.series = sA;
    // ... each configuration keeps its energy
    A.acc[A_ECUR] = ea;
    B.acc[A_ECUR] = eb;
    const int r = perm[k];
    perm[k] = perm[k + 1];
    perm[k + 1] = r;
}

cudaError_t launch_pt_exchange(Rep *reps, int nt, int *perm, unsigned long long seed, long long *acc_cnt,
                               long long *att_cnt, cudaStream_t st)
{
    const int pairs = (nt + 1) / 2;
    k_pt_exchange<<<(pairs + 127) / 128, 128, 0, st>>>(reps, nt, perm, seed, acc_cnt, att_cnt);
    return cudaGetLastError();
}

}  // namespace mcs
