// wp_sim.cu -- seeded read simulator on the GPU (`simulate rad`):
// generate_dye_track (simulation/generate-dye-track.cc:29-110) and
// generate_radiometry (simulation/generate-radiometry.cc:28-62), one thread
// per read, counter-based Philox streams (read r uses subsequence r of the
// seed, so results do not depend on the launch shape).
//
// Per read: a peptide drawn with probability proportional to its count, its
// dyes made duds (per channel p_dud), an initial block, then per timestep:
// record the live dye counts; cyclic block; detach (the read is empty from
// then on); unless blocked, an Edman cycle that succeeds with
// 1 - p_edman_failure and removes the dye at the cut position; bleaching of
// every remaining dye past the cut.  A read whose timestep-0 counts are all
// zero is not detectable and gets peptide index -1 (the reference drops it).
// Intensities are Normal(adjusted_mu, sigma(adjusted_mu)) per (t, c), with
// ChannelModel's interactions (channel-model.h:35-70), drawn in FP64 (in
// FP32 when only FP32 reads are asked for, as for network training).  Each
// Bernoulli event is one 32-bit draw against a precomputed threshold: the
// track part of the kernel does no floating-point work.
//
// With per_peptide > 0 the kernel makes the dye-track instances of the kNN
// training set instead (generate-dye-tracks.cc:32-70): instance r belongs to
// peptide copy r / per_peptide, and only the tracks are written.
//
// The reference draws from std::default_random_engine in a different order,
// so parity with it is statistical (tests compare distributions).
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

#define SIM_MAX_LEN 256


__device__ double sim_adjusted_mu(const DevModel& m, int channel, const int* counts) {
    double amu = m.mu[channel] * (double)counts[channel];
    for (int c = 0; c < m.C; c++) {
        const double fi = m.flat[channel][c], ii = m.inter[channel][c];
        if (c == channel) {
            if (counts[c] > 1) {
                if (fi != 1.0) amu *= fi;
                if (ii != 1.0) amu *= pow(ii, (double)(counts[c] - 1));
            }
        } else if (counts[c] > 0) {
            if (fi != 1.0) amu *= fi;
            if (ii != 1.0) amu *= pow(ii, (double)counts[c]);
        }
    }
    return amu;
}

// The same in FP32, for the FP32 reads the proposal network trains on.
__device__ float sim_adjusted_mu_f(const DevModel& m, int channel, const int* counts) {
    float amu = (float)m.mu[channel] * (float)counts[channel];
    for (int c = 0; c < m.C; c++) {
        const float fi = (float)m.flat[channel][c], ii = (float)m.inter[channel][c];
        const int n = c == channel ? counts[c] - 1 : counts[c];
        if (n > 0) {
            if (fi != 1.0f) amu *= fi;
            if (ii != 1.0f) amu *= powf(ii, (float)n);
        }
    }
    return amu;
}

// bernoulli_distribution(p) with p as a 33-bit threshold; no draw for p = 0.
__device__ __forceinline__ bool sim_event(curandStatePhilox4_32_10_t* st, unsigned long long thr) {
    return thr != 0ull && (unsigned long long)curand(st) < thr;
}

// generate_dye_track for one instance, every labeled position kept as a bit
// of a per-channel 64-bit mask of live dyes (nlab <= 64 labeled positions):
// the live count of a channel is the mask's population, the Edman cut clears
// the bit of the next labeled position when it reaches it, bleaching draws
// once per set bit.  Writes the live counts [T][C] to trk.
__device__ void sim_track_masks(const SimParams& p, curandStatePhilox4_32_10_t* st, const int8_t* seq, int L,
                                int nlab, uint8_t* trk) {
    uint8_t lpos[64];
    uint64_t live[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    int k = 0;
    for (int i = 0; i < L && k < nlab; i++) {
        const int d = seq[i];
        if (d < 0) continue;
        lpos[k] = (uint8_t)i;
        if (!sim_event(st, p.thr_dud[d])) {  // duds
#pragma unroll
            for (int c = 0; c < WP_MAX_CHANNELS; c++)
                if (c == d) live[c] |= 1ull << k;
        }
        k++;
    }
    int e = 0, nk = 0, npos = nlab > 0 ? lpos[0] : L;
    bool block = sim_event(st, p.thr_initial_block), gone = false;
    for (int t = 0; t < p.T; t++) {
        if (!gone && e < L) {
#pragma unroll
            for (int c = 0; c < WP_MAX_CHANNELS; c++)
                if (c < p.C) trk[t * p.C + c] = (uint8_t)__popcll(live[c]);
            if (sim_event(st, p.thr_cyclic_block)) block = true;
            if (sim_event(st, p.thr_detach[t])) {
                gone = true;
                continue;
            }
            if (!block && !sim_event(st, p.thr_fail)) {
                if (e == npos) {  // the cut removes the dye at position e
                    const uint64_t keep = ~(1ull << nk);
#pragma unroll
                    for (int c = 0; c < WP_MAX_CHANNELS; c++) live[c] &= keep;
                    nk++;
                    npos = nk < nlab ? lpos[nk] : L;
                }
                e++;
            }
#pragma unroll
            for (int c = 0; c < WP_MAX_CHANNELS; c++) {  // bleaching past the cut
                uint64_t m = c < p.C ? live[c] : 0ull;
                while (m) {
                    const int b = __ffsll((long long)m) - 1;
                    m &= m - 1;
                    if (sim_event(st, p.thr_bleach[c])) live[c] &= ~(1ull << b);
                }
            }
        } else {
            for (int c = 0; c < p.C; c++) trk[t * p.C + c] = 0;
        }
    }
}

__global__ void wp_sim_reads_kernel(SimParams p) {
    const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p.R) return;
    curandStatePhilox4_32_10_t st;
    curand_init(p.seed, (unsigned long long)r, 0ull, &st);
    // peptide by count weight (upper bound of u * total in the prefix sums),
    // or the peptide of copy r / per_peptide: generate_dye_tracks
    // (generate-dye-tracks.cc:40-47) makes per_peptide tracks for each of
    // the count copies of every dye-seq, in order
    const double total = p.cum[p.P - 1];
    const double u = p.per_peptide > 0 ? (double)(r / p.per_peptide) + 1.0
                                       : curand_uniform_double(&st) * total;  // (0, total]
    int lo = 0, hi = p.P - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (p.cum[mid] >= u) hi = mid;
        else lo = mid + 1;
    }
    const int pep = lo;
    const int L = min(p.offsets[pep + 1] - p.offsets[pep], SIM_MAX_LEN);
    const int8_t* seq = p.seqs + p.offsets[pep];
    __align__(16) uint8_t trk[WP_MAX_TIMESTEPS * WP_MAX_CHANNELS];
    // uploaded dye-seqs carry at most 15 dyes on each of at most 4 channels,
    // so at most 60 labeled positions
    int nlab = 0;
    for (int i = 0; i < L; i++) nlab += seq[i] >= 0;
    sim_track_masks(p, &st, seq, L, min(nlab, 64), trk);
    bool trivial = true;
    for (int c = 0; c < p.C; c++)
        if (trk[c] != 0) trivial = false;
    p.pep[r] = trivial ? -1 : pep;
    const int TC = p.T * p.C;
    if (p.tracks) {
        if (TC % 16 == 0) {  // rows on 16-byte boundaries
            uint4* dst = reinterpret_cast<uint4*>(p.tracks + r * TC);
            for (int q = 0; q < TC / 16; q++) dst[q] = reinterpret_cast<const uint4*>(trk)[q];
        } else {
            for (int i = 0; i < TC; i++) p.tracks[r * TC + i] = trk[i];
        }
    }
    if (!p.rads_f && !p.rads_d) return;  // dye-tracks only
    const DevModel& m = *p.model;
    const bool fp32 = !p.rads_d;  // FP32 reads only: FP32 draws
    for (int t = 0; t < p.T; t++) {
        int cts[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        for (int c = 0; c < p.C; c++) cts[c] = trk[t * p.C + c];
        for (int c = 0; c < p.C; c++) {
            if (fp32) {
                const float mu = sim_adjusted_mu_f(m, c, cts);
                const float bg = (float)m.bg_sig[c], sg1 = (float)m.sig[c];
                const float sg = sqrtf(bg * bg + mu * sg1 * sg1);
                p.rads_f[r * TC + t * p.C + c] = mu + sg * curand_normal(&st);
            } else {
                const double mu = sim_adjusted_mu(m, c, cts);
                const double sg = sqrt(m.bg_sig[c] * m.bg_sig[c] + mu * m.sig[c] * m.sig[c]);
                const double x = mu + sg * curand_normal_double(&st);
                if (p.rads_f) p.rads_f[r * TC + t * p.C + c] = (float)x;
                p.rads_d[r * TC + t * p.C + c] = x;
            }
        }
    }
}

cudaError_t wp_launch_sim_reads(const SimParams& p, cudaStream_t s) {
    if (p.R == 0) return cudaSuccess;
    wp_sim_reads_kernel<<<(p.R + 127) / 128, 128, 0, s>>>(p);
    return cudaGetLastError();
}
