// wp_kernels.cu -- sm_103a kernels of the peptide-HMM forward pass.
//
// Kernels:
//   wp_prep_reads_kernel    one thread per (read, timestep): the emission
//                           pruning box (hmm/step/peptide-emission.cc:50-163)
//                           and the emission factors in FP64, stored as
//                           (FP32 mantissa, int exponent).
//   wp_forward_kernel<B>    one CTA per (read, tile of peptides), one warp per
//                           (read, peptide) pair, the pair's state tensors in
//                           shared memory.  FP32 arithmetic, exact power-of-
//                           two rescaling after every emission, the exponent
//                           kept as an integer (no FP64 in the inner loop).
//   wp_combine_kernel       per read: argmax (first candidate wins ties) and
//                           count-weighted total over its tiles
//                           (classifiers/hmm-classifier.h:45-78).
//   wp_count_flops_kernel   the pruned schedule's visited-state op count.
//
// Pruning.  The reference prunes every step of every pair to an axis-aligned
// box (hmm/hmm/peptide-hmm.cc:63-83).  After both prune passes the box of
// emission t is [L_t, U_t) per channel with L_t = max_{t'>=t} cmin_{t'} and
// U_t = min(D+1, min_{t'<=t} cmax_{t'}), the binomial and Edman boxes follow
// from these, and a pair is empty iff some L_t >= U_t.  Because dye counts
// never increase, computing every state of the pair but zeroing the emission
// factor outside [cmin_t, cmax_t) leaves every state inside the reference's
// boxes unchanged and kills every state outside them before it reaches the
// final sum; the one place where states outside a box would leak is the
// detached-state sum, and the reference drops that sum (allow_detached
// false, peptide-emission.cc:218-223) in exactly the timesteps where it
// would differ.  So the kernels need per-read boxes and allow flags only.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

// ------------------------------------------------------------------ prep --

// ChannelModel::adjusted_mu (parameterization/model/channel-model.h:35-54).
__device__ double dev_adjusted_mu(const DevModel& m, int channel, const unsigned* counts) {
    double amu = m.mu[channel];
    amu *= (double)counts[channel];
    for (int c = 0; c < m.C; c++) {
        if (c == channel) {
            if (counts[c] > 1) {
                amu *= m.flat[channel][c];
                amu *= pow(m.inter[channel][c], (double)(counts[c] - 1));
            }
        } else if (counts[c] > 0) {
            amu *= m.flat[channel][c];
            amu *= pow(m.inter[channel][c], (double)counts[c]);
        }
    }
    return amu;
}

__device__ double dev_sigma(const DevModel& m, int c, double amu) {
    return sqrt(m.bg_sig[c] * m.bg_sig[c] + amu * m.sig[c] * m.sig[c]);
}

// ChannelModel::pdf_helper (channel-model.h:61-70).
__device__ double dev_pdf(const DevModel& m, int c, double observed, const unsigned* counts) {
    const double pi = 3.141592653589793238;
    double amu = dev_adjusted_mu(m, c, counts);
    double offset = observed - amu;
    double s = dev_sigma(m, c, amu);
    return (1.0 / (s * sqrt(2.0 * pi))) * exp(-offset * offset / (2.0 * s * s));
}

__device__ EmitEntry make_entry(double v) {
    EmitEntry e;
    if (v > 0.0 && isfinite(v)) {
        int ex;
        double mant = frexp(v, &ex);
        e.mant = (float)mant;
        e.expo = ex;
        if (e.mant >= 1.0f) {  // rounding up to 1.0
            e.mant = 0.5f;
            e.expo += 1;
        }
    } else {
        e.mant = 0.0f;
        e.expo = WP_EXPO_ZERO;
    }
    return e;
}

// One thread per (read, t).  Writes box_lo/box_hi[r][t][c] and the
// emission entries of timestep t.
__global__ void wp_prep_reads_kernel(const DevModel* __restrict__ model,
                                     const double* __restrict__ rads, int R,
                                     unsigned max_num_dyes, double dist_cutoff,
                                     uint8_t* __restrict__ box_lo,
                                     uint8_t* __restrict__ box_hi,
                                     EmitEntry* __restrict__ table, int entries_per_read) {
    const DevModel& m = *model;
    const int T = m.T, C = m.C;
    long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)R * T) return;
    int r = (int)(gid / T), t = (int)(gid % T);
    const double* rad = rads + (long)r * T * C;
    unsigned lo[WP_MAX_CHANNELS], hi[WP_MAX_CHANNELS];
    // PeptideEmission ctor pruned_range (peptide-emission.cc:50-163).
    if (dist_cutoff == DBL_MAX) {
        for (int c = 0; c < C; c++) {
            lo[c] = 0;
            hi[c] = max_num_dyes + 1;
        }
    } else {
        unsigned counts_lo[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        unsigned counts_hi[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        bool did_change = true;
        int guard = 0;
        // The reference loops to a fixed point without a bound and cycles
        // forever for intensities below about -0.5 mu; stop after 1000
        // rounds (the oracle uses the same bound).
        while (did_change && guard < 1000) {
            did_change = false;
            guard++;
            for (int c = 0; c < C; c++) {
                unsigned old = counts_hi[c];
                counts_hi[c] = 1;
                double mu1 = dev_adjusted_mu(m, c, counts_hi);
                counts_hi[c] = old;
                double mu = dev_adjusted_mu(m, c, counts_hi);
                double s = dist_cutoff * dev_sigma(m, c, mu);
                unsigned new_cts = (unsigned)lround((rad[t * C + c] + s) / mu1);
                if (new_cts > max_num_dyes + 1) new_cts = max_num_dyes + 1;
                if (new_cts != counts_hi[c]) {
                    did_change = true;
                    counts_hi[c] = new_cts;
                }
            }
        }
        for (int c = 0; c < C; c++) {
            unsigned cmin = max_num_dyes + 1;
            for (unsigned d = 0; d < max_num_dyes + 1; d++) {
                counts_lo[c] = d;
                double mu = dev_adjusted_mu(m, c, counts_lo);
                double s = dist_cutoff * dev_sigma(m, c, mu);
                if (mu + s > rad[t * C + c]) {
                    cmin = d;
                    break;
                }
            }
            counts_lo[c] = 0;
            unsigned cmax = max_num_dyes + 1;
            unsigned old = counts_hi[c];
            for (unsigned d = cmin; d < max_num_dyes + 1; d++) {
                counts_hi[c] = d;
                double mu = dev_adjusted_mu(m, c, counts_hi);
                double s = dist_cutoff * dev_sigma(m, c, mu);
                if (mu - s > rad[t * C + c]) {
                    cmax = d;
                    break;
                }
            }
            counts_hi[c] = old;
            lo[c] = cmin;
            hi[c] = cmax;
        }
    }
    for (int c = 0; c < C; c++) {
        box_lo[((long)r * T + t) * C + c] = (uint8_t)lo[c];
        box_hi[((long)r * T + t) * C + c] = (uint8_t)hi[c];
    }
    // Emission factors (peptide-emission.cc:167-180): the product over
    // channels of the Gaussian pdf, zero outside the box.
    const int W = (int)max_num_dyes + 1;
    EmitEntry* out = table + (long)r * entries_per_read;
    if (!m.interacting) {
        // pdf of channel c depends on n_c only: store per (t, c, n).
        for (int c = 0; c < C; c++) {
            for (int n = 0; n < W; n++) {
                double v = 0.0;
                if ((unsigned)n >= lo[c] && (unsigned)n < hi[c]) {
                    unsigned counts[WP_MAX_CHANNELS] = {0, 0, 0, 0};
                    counts[c] = (unsigned)n;
                    v = dev_pdf(m, c, rad[t * C + c], counts);
                }
                out[(t * C + c) * W + n] = make_entry(v);
            }
        }
    } else {
        int G = wp_ipow(W, C);
        for (int g = 0; g < G; g++) {
            unsigned counts[WP_MAX_CHANNELS] = {0, 0, 0, 0};
            int rem = g;
            bool in_box = true;
            for (int c = C - 1; c >= 0; c--) {
                counts[c] = (unsigned)(rem % W);
                rem /= W;
                if (counts[c] < lo[c] || counts[c] >= hi[c]) in_box = false;
            }
            double v = 0.0;
            if (in_box) {
                v = 1.0;
                for (int c = 0; c < C; c++) v *= dev_pdf(m, c, rad[t * C + c], counts);
            }
            out[t * G + g] = make_entry(v);
        }
    }
}

// --------------------------------------------------------------- forward --

// 2^x as a float for x <= 127 (0 below the subnormal range).
__device__ __forceinline__ float exp2i(int x) {
    if (x >= -126) return __int_as_float((min(x, 127) + 127) << 23);
    if (x >= -149) return ldexpf(1.0f, x);
    return 0.0f;
}



#define WP_TILE_MAX 1024
#define WP_FWD_WARPS_MAX 16

struct SmemHead {
    float dud[WP_MAX_CHANNELS][WP_TRI];
    float bleach[WP_MAX_CHANNELS][WP_TRI];
    float p_det[WP_MAX_TIMESTEPS];
    uint8_t lo[WP_MAX_TIMESTEPS][WP_MAX_CHANNELS];
    uint8_t hi[WP_MAX_TIMESTEPS][WP_MAX_CHANNELS];
    // Non-interacting: max exponent over [lo, min(hi, u)) per (t, c, u).
    int pmk[WP_MAX_TIMESTEPS][WP_MAX_CHANNELS][WP_W + 1];
    uint8_t allow[WP_MAX_TIMESTEPS];
    uint8_t minD[WP_MAX_CHANNELS];
    int read_empty;
    int next;
    float res_mant[WP_TILE_MAX];
    int res_expo[WP_TILE_MAX];
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ int warp_max_int(int v) {
    return __reduce_max_sync(0xffffffffu, v);
}

// In-place binomial transition along one channel axis for every fiber of
// the slices e < e_count (binomial-transition.cc:114-136):
// out[to] = sum_{from >= to} prob(from, to) * in[from].
template <int W>
__device__ void binomial_fibers(float* X, int S, int F, int nf, int stc,
                                const uint16_t* __restrict__ fib,
                                const float* __restrict__ tab, int lane) {
    float p[W * (W + 1) / 2];
#pragma unroll
    for (int i = 0; i < W * (W + 1) / 2; i++) p[i] = tab[i];
    int e = lane / F, r = lane - (lane / F) * F;
    const int de = 32 / F, dr = 32 - de * F;
    for (int f = lane; f < nf; f += 32) {
        int base = e * S + fib[r];
        float v[W];
#pragma unroll
        for (int i = 0; i < W; i++) v[i] = X[base + i * stc];
#pragma unroll
        for (int to = 0; to < W; to++) {
            float acc = 0.0f;
#pragma unroll
            for (int from = to; from < W; from++) acc = fmaf(p[from * (from + 1) / 2 + to], v[from], acc);
            X[base + to * stc] = acc;
        }
        r += dr;
        e += de;
        if (r >= F) {
            r -= F;
            e++;
        }
    }
}

// Same transition for W > 8: table entries read from shared memory (one
// broadcast load per multiply-add), in place with ascending `to`.
__device__ void binomial_fibers_wide(float* X, int S, int W, int F, int nf, int stc,
                                     const uint16_t* __restrict__ fib,
                                     const float* __restrict__ tab, int lane) {
    int e = lane / F, r = lane - (lane / F) * F;
    const int de = 32 / F, dr = 32 - de * F;
    for (int f = lane; f < nf; f += 32) {
        int base = e * S + fib[r];
        for (int to = 0; to < W; to++) {
            float acc = 0.0f;
            for (int from = to; from < W; from++)
                acc = fmaf(tab[from * (from + 1) / 2 + to], X[base + from * stc], acc);
            X[base + to * stc] = acc;
        }
        r += dr;
        e += de;
        if (r >= F) {
            r -= F;
            e++;
        }
    }
}

__device__ void binomial_step(float* X, int S, int W, int e_count, int stc,
                              const uint16_t* fib, const float* tab, int lane) {
    int F = S / W;
    int nf = e_count * F;
    switch (W) {
#define WP_BCASE(w) case w: binomial_fibers<w>(X, S, F, nf, stc, fib, tab, lane); break;
        WP_BCASE(2) WP_BCASE(3) WP_BCASE(4) WP_BCASE(5) WP_BCASE(6) WP_BCASE(7) WP_BCASE(8)
#undef WP_BCASE
        default: binomial_fibers_wide(X, S, W, F, nf, stc, fib, tab, lane); break;
    }
}

// Per-warp shared memory carve-up.
struct WarpBufs {
    float* X;
    float* Y;
    float* XB;
    float* YB;
    float* em;
    uint16_t* coord;
    uint16_t* fib;  // [C][S_cap]
};

__host__ __device__ inline size_t wp_warp_bytes(int T, int S_cap, int C, bool has_block) {
    size_t f = (size_t)(has_block ? 4 : 2) * T * S_cap + S_cap;
    size_t h = (size_t)S_cap * (1 + C);
    size_t b = f * 4 + h * 2;
    return (b + 15) & ~(size_t)15;
}

// Forward pass of one (read, peptide) pair by one warp.  Returns the
// probability as mant * 2^expo (mant == 0: probability zero).
template <bool HAS_BLOCK>
__device__ void pair_forward(const SmemHead& H, const EmitEntry* __restrict__ rtab,
                             const DevModel& m, const PeptideRec& pep, int W_read,
                             const WarpBufs& wb, int S_cap, int lane,
                             float* out_mant, int* out_expo, int* err) {
    const int C = m.C, T = m.T;
    int Wc[WP_MAX_CHANNELS], st[WP_MAX_CHANNELS];
    int S = 1;
    bool empty = H.read_empty != 0;
    for (int c = 0; c < C; c++) {
        Wc[c] = pep.D[c] + 1;
        if (pep.D[c] < H.minD[c]) empty = true;  // some L_t > D_c
    }
    for (int c = C - 1; c >= 0; c--) {
        st[c] = S;
        S *= Wc[c];
    }
    if (empty) {
        *out_mant = 0.0f;
        *out_expo = 0;
        return;
    }
    if (S > S_cap) {
        if (lane == 0) atomicExch(err, 1);
        *out_mant = 0.0f;
        *out_expo = 0;
        return;
    }
    // Coordinates of each state of an Edman slice, 4 bits per channel.
    for (int j = lane; j < S; j += 32) {
        int code = 0;
        for (int c = 0; c < C; c++) code |= ((j / st[c]) % Wc[c]) << (4 * c);
        wb.coord[j] = (uint16_t)code;
    }
    // Fiber base offsets per channel: the states with n_c == 0.
    for (int c = 0; c < C; c++) {
        if (Wc[c] == 1) continue;
        int F = S / Wc[c];
        for (int rr = lane; rr < F; rr += 32) {
            int rem = rr, j = 0;
            for (int c2 = C - 1; c2 >= 0; c2--) {
                if (c2 == c) continue;
                j += (rem % Wc[c2]) * st[c2];
                rem /= Wc[c2];
            }
            wb.fib[c * S_cap + rr] = (uint16_t)j;
        }
    }
    float* X = wb.X;
    float* Y = wb.Y;
    float* XB = wb.XB;
    float* YB = wb.YB;
    // t = 0: start state (0, D) (peptide-state-vector.cc:38-40), initial
    // block (block-transition.cc:33-62), then duds per channel.
    for (int j = lane; j < S; j += 32) {
        float a = (j == S - 1) ? 1.0f : 0.0f;
        if (HAS_BLOCK) {
            XB[j] = m.p_ib * a;
            a = (1.0f - m.p_ib) * a;
        }
        X[j] = a;
    }
    __syncwarp();
    for (int c = 0; c < C; c++) {
        if (Wc[c] == 1) continue;
        binomial_step(X, S, Wc[c], 1, st[c], wb.fib + c * S_cap, H.dud[c], lane);
        if (HAS_BLOCK) binomial_step(XB, S, Wc[c], 1, st[c], wb.fib + c * S_cap, H.dud[c], lane);
        __syncwarp();
    }
    int expo = 0;       // log2 of the factor the stored state is scaled by
    float pd = 0.0f;    // detached state, in the rescaled frame
    int k_prev = 0;     // exponent removed at the last rescale
    float fac_prev = 1.0f;  // (1 - p_detach) pending from the last timestep
    for (int t = 0; t < T; t++) {
        if (t > 0) {
            // Cyclic block (block-transition.cc:33-62).
            if (HAS_BLOCK) {
                int n = t * S;
                for (int i = lane; i < n; i += 32) {
                    float a = X[i];
                    XB[i] = XB[i] + m.p_cb * a;
                    X[i] = (1.0f - m.p_cb) * a;
                }
                __syncwarp();
            }
            // Detach (detach-transition.cc:36-68) is folded into the
            // previous rescale (pd) and the pending factor fac_prev.
            // Bleach per channel.
            for (int c = 0; c < C; c++) {
                if (Wc[c] == 1) continue;
                binomial_step(X, S, Wc[c], t, st[c], wb.fib + c * S_cap, H.bleach[c], lane);
                if (HAS_BLOCK) binomial_step(XB, S, Wc[c], t, st[c], wb.fib + c * S_cap, H.bleach[c], lane);
                __syncwarp();
            }
            // Edman (edman-transition.cc:62-162) as a gather into Y.
            {
                const float pf = m.pf, qf = 1.0f - m.pf;
                int n = (t + 1) * S;
                int e = lane / S, j = lane - (lane / S) * S;
                const int de = 32 / S, dj = 32 - de * S;
                for (int i = lane; i < n; i += 32) {
                    float v = 0.0f;
                    if (e < t) v = pf * X[i];
                    if (e >= 1) {
                        int c = pep.dye[e - 1];
                        float xin = X[i - S];
                        if (c < 0) {
                            v = fmaf(qf, xin, v);
                        } else {
                            int nc = (wb.coord[j] >> (4 * c)) & 15;
                            float tot = (float)pep.tot[e - 1];
                            float ratio = (float)nc / tot;
                            if (nc < pep.tot[e - 1]) v = fmaf(qf * (1.0f - ratio), xin, v);
                            if (nc + 1 < Wc[c]) {
                                float r1 = (float)(nc + 1) / tot;
                                v = fmaf(qf * r1, X[i - S + st[c]], v);
                            }
                        }
                    }
                    Y[i] = v;
                    if (HAS_BLOCK) YB[i] = (e < t) ? XB[i] : 0.0f;
                    j += dj;
                    e += de;
                    if (j >= S) {
                        j -= S;
                        e++;
                    }
                }
                float* tmp = X;
                X = Y;
                Y = tmp;
                if (HAS_BLOCK) {
                    tmp = XB;
                    XB = YB;
                    YB = tmp;
                }
                __syncwarp();
            }
        }
        // Emission factors of this timestep for this pair, normalised by the
        // largest exponent over the pair's reachable box.
        int kmax;
        if (!m.interacting) {
            kmax = 0;
            for (int c = 0; c < C; c++) {
                int km = H.pmk[t][c][Wc[c]];
                if (km == WP_EXPO_ZERO) kmax = WP_EXPO_ZERO;
                if (kmax != WP_EXPO_ZERO) kmax += km;
            }
        } else {
            int km = WP_EXPO_ZERO;
            for (int j = lane; j < S; j += 32) {
                int code = wb.coord[j], g = 0;
                for (int c = 0; c < C; c++) g = g * W_read + ((code >> (4 * c)) & 15);
                EmitEntry en = rtab[t * wp_ipow(W_read, C) + g];
                if (en.mant != 0.0f) km = max(km, en.expo);
            }
            kmax = warp_max_int(km);
        }
        if (kmax == WP_EXPO_ZERO) {  // no reachable state emits
            *out_mant = 0.0f;
            *out_expo = 0;
            return;
        }
        float em0 = 0.0f;
        for (int j = lane; j < S; j += 32) {
            int code = wb.coord[j];
            float mant = 1.0f;
            int ks = 0;
            if (!m.interacting) {
                for (int c = 0; c < C; c++) {
                    EmitEntry en = rtab[(t * C + c) * W_read + ((code >> (4 * c)) & 15)];
                    mant *= en.mant;
                    ks += en.expo;
                }
            } else {
                int g = 0;
                for (int c = 0; c < C; c++) g = g * W_read + ((code >> (4 * c)) & 15);
                EmitEntry en = rtab[t * wp_ipow(W_read, C) + g];
                mant = en.mant;
                ks = en.expo;
            }
            float ev = 0.0f;
            if (mant != 0.0f) {
                int d = ks - kmax;
                if (j == 0) em0 = mant * exp2i(max(d, -200));
                ev = (mant * fac_prev) * exp2i(max(min(d - k_prev, 127), -200));
            }
            wb.em[j] = ev;
        }
        em0 = __shfl_sync(0xffffffffu, em0, 0);
        __syncwarp();
        // Emission (peptide-emission.cc:212-243) over e <= t, with the
        // pending rescale folded in, and the state sum.
        float part = 0.0f;
        {
            int n = (t + 1) * S;
            int j = lane % S;
            const int dj = 32 % S;
            for (int i = lane; i < n; i += 32) {
                float w = wb.em[j];
                float a = X[i] * w;
                X[i] = a;
                part += a;
                if (HAS_BLOCK) {
                    float b = XB[i] * w;
                    XB[i] = b;
                    part += b;
                }
                j += dj;
                if (j >= S) j -= S;
            }
        }
        // The butterfly leaves lane-dependent rounding; take lane 0's value so
        // that every lane applies the same rescale.
        float sum_ab = __shfl_sync(0xffffffffu, warp_sum(part), 0);
        pd = H.allow[t] ? pd * em0 : 0.0f;
        expo += kmax;
        float tot = sum_ab + pd;
        if (!(tot > 0.0f) || !isfinite(tot)) {
            *out_mant = 0.0f;
            *out_expo = 0;
            return;
        }
        int k;
        float fm = frexpf(tot, &k);
        if (t == T - 1) {
            *out_mant = fm;
            *out_expo = expo + k;
            return;
        }
        float f = exp2i(-k);
        expo += k;
        // Detach of the next timestep (detach-transition.cc:36-68), in the
        // rescaled frame; the stored state keeps its scale until the next
        // emission multiplies in f * (1 - p_detach).
        pd = (pd + H.p_det[t] * sum_ab) * f;
        k_prev = k;
        fac_prev = 1.0f - H.p_det[t];
        __syncwarp();
    }
}

// A probability mant * 2^expo (mant in [0.5, 1) or 0) with its tie key.
struct Cand {
    float mant;
    int expo;
    int key;
    int idx;  // < 0: no candidate
};

// True if a beats b: larger probability, then smaller key (the reference's
// strict '>' over candidates in order, classifiers/hmm-classifier.h:62).
__device__ __forceinline__ bool cand_better(const Cand& a, const Cand& b) {
    if (a.idx < 0) return false;
    if (b.idx < 0) return true;
    bool az = a.mant == 0.0f, bz = b.mant == 0.0f;
    if (az && bz) return a.key < b.key;
    if (az) return false;
    if (bz) return true;
    if (a.expo != b.expo) return a.expo > b.expo;
    if (a.mant != b.mant) return a.mant > b.mant;
    return a.key < b.key;
}

template <bool HAS_BLOCK>
__global__ void __launch_bounds__(WP_FWD_WARPS_MAX * 32)
wp_forward_kernel(TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemHead& H = *reinterpret_cast<SmemHead*>(smem_raw);
    const DevModel& m = *a.model;
    const int C = m.C, T = m.T;
    const int tile = blockIdx.x;
    const int r = a.tile_read[tile];
    const int begin = a.tile_begin[tile], end = a.tile_end[tile];
    const int n_items = end - begin;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const EmitEntry* rtab = a.table + (long)r * a.entries;

    // Model tables.
    for (int i = threadIdx.x; i < C * WP_TRI; i += blockDim.x) {
        int c = i / WP_TRI, k = i % WP_TRI;
        H.dud[c][k] = m.dud[c][k];
        H.bleach[c][k] = m.bleach[c][k];
    }
    for (int t = threadIdx.x; t < T; t += blockDim.x) H.p_det[t] = m.p_det[t];
    for (int i = threadIdx.x; i < T * C; i += blockDim.x) {
        H.lo[i / C][i % C] = a.box_lo[(long)r * T * C + i];
        H.hi[i / C][i % C] = a.box_hi[(long)r * T * C + i];
    }
    if (threadIdx.x == 0) H.next = 0;
    __syncthreads();
    // Per (t, c): running max of the exponent over [lo, min(hi, u)).
    if (!m.interacting) {
        for (int i = threadIdx.x; i < T * C; i += blockDim.x) {
            int t = i / C, c = i % C;
            int run = WP_EXPO_ZERO;
            H.pmk[t][c][0] = run;
            for (int u = 1; u <= WP_W; u++) {
                int n = u - 1;
                if (n < a.W && n >= H.lo[t][c] && n < H.hi[t][c]) {
                    EmitEntry en = rtab[(t * C + c) * a.W + n];
                    if (en.mant != 0.0f) run = max(run, en.expo);
                }
                H.pmk[t][c][u] = run;
            }
        }
    }
    // Read-level pruning summary: L_t (suffix max of cmin), U_t (prefix min
    // of cmax), allow_detached per emission, emptiness, min dyes per channel.
    if (threadIdx.x == 0) {
        int L[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        int empty = 0;
        for (int t = T - 1; t >= 0; t--) {
            int allow = 1;
            for (int c = 0; c < C; c++) {
                L[c] = max(L[c], (int)H.lo[t][c]);
                if (L[c] != 0) allow = 0;
            }
            H.allow[t] = (uint8_t)allow;
        }
        for (int c = 0; c < C; c++) H.minD[c] = (uint8_t)L[c];
        int U[WP_MAX_CHANNELS] = {255, 255, 255, 255};
        int Lt[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        // recompute suffix max per t to test emptiness L_t >= U_t
        for (int t = 0; t < T; t++) {
            for (int c = 0; c < C; c++) {
                U[c] = min(U[c], (int)H.hi[t][c]);
                int l = 0;
                for (int t2 = t; t2 < T; t2++) l = max(l, (int)H.lo[t2][c]);
                Lt[c] = l;
                if (Lt[c] >= U[c]) empty = 1;
                if (U[c] == 0) H.allow[t] = 0;
            }
        }
        H.read_empty = empty;
    }
    __syncthreads();

    // Per-warp buffers.
    unsigned char* wbase = smem_raw + ((sizeof(SmemHead) + 15) & ~(size_t)15);
    size_t wbytes = wp_warp_bytes(T, a.S_cap, C, HAS_BLOCK);
    float* fb = reinterpret_cast<float*>(wbase + wbytes * warp);
    WarpBufs wb;
    size_t slab = (size_t)T * a.S_cap;
    wb.X = fb;
    wb.Y = fb + slab;
    float* after = fb + 2 * slab;
    if (HAS_BLOCK) {
        wb.XB = fb + 2 * slab;
        wb.YB = fb + 3 * slab;
        after = fb + 4 * slab;
    } else {
        wb.XB = wb.YB = nullptr;
    }
    wb.em = after;
    wb.coord = reinterpret_cast<uint16_t*>(after + a.S_cap);
    wb.fib = wb.coord + a.S_cap;

    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(&H.next, 1);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n_items) break;
        int p = a.list[begin + idx];
        const PeptideRec& pep = a.peps[p];
        float mant;
        int ex;
        pair_forward<HAS_BLOCK>(H, rtab, m, pep, a.W, wb, a.S_cap, lane, &mant, &ex, a.err);
        if (lane == 0) {
            if (a.out_logp) {
                a.out_logp[(long)r * a.num_peptides + p] =
                        mant > 0.0f ? log((double)mant) + (double)ex * 0.69314718055994530942 : -INFINITY;
            }
            if (idx < WP_TILE_MAX) {
                H.res_mant[idx] = mant;
                H.res_expo[idx] = mant > 0.0f ? ex : 0;
            }
        }
        __syncwarp();
    }
    __syncthreads();
    // Tile reduction: best (largest P, smallest key on ties) and the
    // count-weighted total relative to the best's exponent.  Deterministic:
    // fixed lane assignment and a fixed butterfly.
    if (a.part_key && warp == 0) {
        Cand best = {0.0f, 0, INT_MAX, -1};
        for (int i = lane; i < n_items; i += 32) {
            Cand c = {H.res_mant[i], H.res_expo[i], a.key[begin + i], i};
            if (cand_better(c, best)) best = c;
        }
        for (int o = 16; o > 0; o >>= 1) {
            Cand c;
            c.mant = __shfl_xor_sync(0xffffffffu, best.mant, o);
            c.expo = __shfl_xor_sync(0xffffffffu, best.expo, o);
            c.key = __shfl_xor_sync(0xffffffffu, best.key, o);
            c.idx = __shfl_xor_sync(0xffffffffu, best.idx, o);
            if (cand_better(c, best)) best = c;
        }
        int ref_e = (best.mant > 0.0f) ? best.expo : 0;
        double tot = 0.0;
        for (int i = lane; i < n_items; i += 32) {
            float mm = H.res_mant[i];
            if (mm > 0.0f) {
                int p = a.list[begin + i];
                tot += (double)a.counts[p] * ldexp((double)mm, H.res_expo[i] - ref_e);
            }
        }
        for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
        if (lane == 0) {
            const int o = a.tile_out[tile];
            a.part_key[o] = best.idx >= 0 ? best.key : INT_MAX;
            a.part_pep[o] = best.idx >= 0 ? a.list[begin + best.idx] : -1;
            a.part_mant[o] = best.mant;
            a.part_expo[o] = ref_e;
            a.part_total[o] = tot;
        }
    }
}

template __global__ void wp_forward_kernel<false>(TileArgs);
template __global__ void wp_forward_kernel<true>(TileArgs);

size_t wp_forward_smem_bytes(int T, int S_cap, int C, bool has_block, int warps) {
    return ((sizeof(SmemHead) + 15) & ~(size_t)15) + wp_warp_bytes(T, S_cap, C, has_block) * warps;
}

cudaError_t wp_launch_forward(bool has_block, int grid, int threads, size_t smem,
                              cudaStream_t stream, const TileArgs& args) {
    cudaError_t e;
    if (has_block) {
        e = cudaFuncSetAttribute(wp_forward_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        wp_forward_kernel<true><<<grid, threads, smem, stream>>>(args);
    } else {
        e = cudaFuncSetAttribute(wp_forward_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        wp_forward_kernel<false><<<grid, threads, smem, stream>>>(args);
    }
    return cudaGetLastError();
}

// --------------------------------------------------------------- combine --

// Per read: combine its tiles (read_tile_off[r] .. read_tile_off[r+1]) into
// (id, score, total) with the reference's tie rule and NaN patch.
__global__ void wp_combine_kernel(int R, const int* __restrict__ read_tile_off,
                                  const int* __restrict__ part_key,
                                  const int* __restrict__ part_pep,
                                  const float* __restrict__ part_mant,
                                  const int* __restrict__ part_expo,
                                  const double* __restrict__ part_total,
                                  const int* __restrict__ pep_ids,
                                  int32_t* __restrict__ out_id, double* __restrict__ out_score,
                                  double* __restrict__ out_total, double* __restrict__ out_log) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    int b = read_tile_off[r], e = read_tile_off[r + 1];
    int bi = -1;
    for (int k = b; k < e; k++) {
        if (part_pep[k] < 0) continue;
        if (bi < 0) {
            bi = k;
            continue;
        }
        float m1 = part_mant[k], m0 = part_mant[bi];
        bool better;
        if (m1 == 0.0f && m0 == 0.0f) better = part_key[k] < part_key[bi];
        else if (m1 == 0.0f) better = false;
        else if (m0 == 0.0f) better = true;
        else if (part_expo[k] != part_expo[bi]) better = part_expo[k] > part_expo[bi];
        else if (m1 != m0) better = m1 > m0;
        else better = part_key[k] < part_key[bi];
        if (better) bi = k;
    }
    if (bi < 0) {
        out_id[r] = -1;
        out_score[r] = 0.0;
        out_total[r] = 1.0;
        if (out_log) out_log[r] = -INFINITY;
        return;
    }
    int E = part_expo[bi];
    double tot = 0.0;
    for (int k = b; k < e; k++)
        if (part_pep[k] >= 0) tot += ldexp(part_total[k], part_expo[k] - E);
    double sc = (double)part_mant[bi];
    out_id[r] = pep_ids[part_pep[bi]];
    if (!(tot > 0.0) || isnan(sc / tot)) {
        // HMMClassifier's NaN patch (classifiers/hmm-classifier.h:73-76).
        out_score[r] = 0.0;
        out_total[r] = 1.0;
        if (out_log) out_log[r] = -INFINITY;
        return;
    }
    double s_abs = ldexp(sc, E), t_abs = ldexp(tot, E);
    if (s_abs > 0.0 && isfinite(s_abs) && isfinite(t_abs) && s_abs >= DBL_MIN) {
        out_score[r] = s_abs;
        out_total[r] = t_abs;
    } else {
        out_score[r] = sc;
        out_total[r] = tot;
    }
    if (out_log) out_log[r] = log(sc) + (double)E * 0.69314718055994530942;
}

// ---------------------------------------------------------------- flops --

// Visited-state operation count of the reference's pruned schedule for one
// pair, from the closed-form boxes (see the header comment).  One thread per
// (read, peptide).  Sums per read into out[r] (exact: integers < 2^53).
__global__ void wp_count_flops_kernel(const DevModel* __restrict__ model,
                                      const PeptideRec* __restrict__ peps, int P,
                                      const uint8_t* __restrict__ box_lo,
                                      const uint8_t* __restrict__ box_hi, int R,
                                      double* __restrict__ out) {
    const DevModel& m = *model;
    const int T = m.T, C = m.C;
    long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)R * P) return;
    int r = (int)(gid / P), p = (int)(gid % P);
    const uint8_t* lo = box_lo + (long)r * T * C;
    const uint8_t* hi = box_hi + (long)r * T * C;
    const PeptideRec& pep = peps[p];
    int L[WP_MAX_TIMESTEPS][WP_MAX_CHANNELS], U[WP_MAX_TIMESTEPS][WP_MAX_CHANNELS];
    for (int c = 0; c < C; c++) {
        int l = 0;
        for (int t = T - 1; t >= 0; t--) {
            l = max(l, (int)lo[t * C + c]);
            L[t][c] = l;
        }
        int u = pep.D[c] + 1;
        for (int t = 0; t < T; t++) {
            u = min(u, (int)hi[t * C + c]);
            U[t][c] = u;
        }
    }
    for (int t = 0; t < T; t++)
        for (int c = 0; c < C; c++)
            if (L[t][c] >= U[t][c]) return;  // empty: no work
    double fl = 0.0;
    // t = 0
    {
        double vol_init = 1.0, vol_emit = 1.0;
        for (int c = 0; c < C; c++) {
            vol_init *= (double)(pep.D[c] + 1 - L[0][c]);
            vol_emit *= (double)(U[0][c] - L[0][c]);
        }
        if (m.p_ib != 0.0f) fl += 3.0 * vol_init;
        for (int c = 0; c < C; c++) {
            double fibers = 1.0;
            for (int c2 = 0; c2 < C; c2++) {
                if (c2 == c) continue;
                fibers *= (c2 < c) ? (double)(U[0][c2] - L[0][c2]) : (double)(pep.D[c2] + 1 - L[0][c2]);
            }
            double macs = 0.0;
            for (int to = L[0][c]; to < U[0][c]; to++) macs += (double)(pep.D[c] + 1 - to);
            fl += 2.0 * fibers * macs;
        }
        fl += 1.0 * vol_emit + 2.0 * vol_emit;
    }
    for (int t = 1; t < T; t++) {
        double vol_prev = 1.0, vol_bt = 1.0, vol_next = 1.0;
        int Bt[WP_MAX_CHANNELS];
        for (int c = 0; c < C; c++) {
            Bt[c] = min(U[t][c] + 1, U[t - 1][c]);
            vol_prev *= (double)(U[t - 1][c] - L[t - 1][c]);
            vol_bt *= (double)(Bt[c] - L[t][c]);
            vol_next *= (double)(U[t][c] - L[t][c]);
        }
        if (m.p_cb != 0.0f) fl += 3.0 * t * vol_prev;
        fl += 2.0 * t * vol_prev;  // detach
        for (int c = 0; c < C; c++) {
            double fibers = (double)t;
            for (int c2 = 0; c2 < C; c2++) {
                if (c2 == c) continue;
                fibers *= (c2 < c) ? (double)(Bt[c2] - L[t][c2]) : (double)(U[t - 1][c2] - L[t - 1][c2]);
            }
            double macs = 0.0;
            for (int to = L[t][c]; to < Bt[c]; to++) {
                int from_min = max(to, L[t - 1][c]);
                if (U[t - 1][c] > from_min) macs += (double)(U[t - 1][c] - from_min);
            }
            fl += 2.0 * fibers * macs;
        }
        fl += 6.0 * t * vol_bt;             // Edman
        fl += 3.0 * (t + 1) * vol_next;     // emission + rescale
    }
    atomicAdd(&out[r], fl);
}

// ------------------------------------------------------------ FP32 peak --

// Eight independent FMA chains per thread; the result is stored so that the
// chains are not removed.  2 flops per FMA.
__global__ void wp_fma_probe_kernel(int iters, float* sink) {
    float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    float a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const float b = 0.999f, c = 1e-3f;
    for (int i = 0; i < iters; i++) {
        a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
        a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

cudaError_t wp_launch_fma_probe(int blocks, int threads, int iters, cudaStream_t stream, float* sink) {
    wp_fma_probe_kernel<<<blocks, threads, 0, stream>>>(iters, sink);
    return cudaGetLastError();
}
