// wp_prep.cu -- per-read preparation and pair compaction.
//
//   wp_prep_reads_kernel    one thread per (read, timestep): the emission
//                           pruning box [cmin, cmax) of the reference's
//                           PeptideEmission (hmm/step/peptide-emission.cc:
//                           50-163), in FP64 as the reference computes it
//                           (without interactions from per-CTA tables of
//                           its thresholds), and the emission factors,
//                           stored as (FP32 mantissa, int exponent) of
//                           norm * 2^y with y in FP64 (the FP64 exp only in
//                           the far tails).
//   wp_read_summary_kernel  one thread per read: the closed-form pruning boxes
//                           every pair of the read shares, L_t = max_{t'>=t}
//                           cmin_{t'} and min_{t'<=t} cmax_{t'}, the
//                           allow-detached flag of each emission and whether
//                           the read prunes every pair.
//   wp_window_factors_kernel  one thread per (read, timestep): the emission
//                           factors normalised over the pruning window, for
//                           the engine (non-interacting models); the CTA's
//                           rows staged through shared memory.
//   wp_compact_kernel       one CTA per read (candidate lists, loglik):
//                           pairs whose pruned range is empty get
//                           probability 0 (PeptideHMM::probability,
//                           hmm/hmm/peptide-hmm.cc:94-100); the others are
//                           appended to the work list of the first engine
//                           pass whose per-thread slab holds their largest
//                           box (pair_vmax), or to the dense kernel's list.
//   wp_compact_groups_kernel  the same for classify over all peptides, one
//                           warp per read and one decision per group of
//                           peptides with one dye-count vector, the groups
//                           appended in the order of their counts clamped to
//                           the read's bounds (pairs that take the same
//                           steps side by side); empty pairs get no write.
//
// Pruning.  After the reference's forward and backward prune passes
// (hmm/hmm/peptide-hmm.cc:63-83) the box of emission t of a pair is
// [L_t, U_t) per channel with L_t = max_{t'>=t} cmin_{t'} and
// U_t = min(D + 1, min_{t'<=t} cmax_{t'}) (D = the pair's dyes on that
// channel); the binomial and Edman steps in between use the boxes derived
// from these two; the pair is empty iff some L_t >= U_t, i.e. iff the read is
// empty on its own or L_0 > D on some channel.  tests/test_oracle.py checks
// this closed form against the literal prune passes of the oracle.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

#define WP_COMPACT_SORT 1024  // candidate slots per read the compaction orders by shape
#define WP_COMPACT_UNIQ 1024  // distinct dye-count vectors the compaction tabulates per read
#define WP_COMPACT_CHUNK 2048  // slots the compaction routes per round of list appends
#define WP_GROUP_BUCKETS 512  // clamped dye-count vectors the group compaction counting-sorts per read
static_assert(WP_GROUP_BUCKETS >= WP_GROUP_MAX, "the group compaction lists its runs in the buckets");


// ChannelModel::adjusted_mu (parameterization/model/channel-model.h:35-54).
__device__ double dev_adjusted_mu(const DevModel& m, int channel, const unsigned* counts) {
    double amu = m.mu[channel];
    amu *= (double)counts[channel];
    for (int c = 0; c < m.C; c++) {
        // A factor of exactly 1 leaves amu unchanged (pow(1, n) == 1 and
        // x * 1 == x), so the common no-interaction case skips the pow.
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
    const bool tabled = !m.interacting;  // per-count quantities from the model's tables
    // Non-interacting models: the pruning thresholds mu_d + s_d and mu_d -
    // s_d (s_d = dist_cutoff * sigma_d) per (channel, count), once per CTA,
    // each rounded as the reference's separate multiply and add round it.
    // And the pdf's normalisation 1 / (sigma sqrt(2 pi)) as an FP32
    // mantissa in [0.5, 1) and an exponent.
    // The thresholds also rounded to FP32 (rounding is monotone, so FP32
    // order decides every comparison but ties, which go to FP64), and
    // log2(e) / (2 sigma^2) times 2^40 (exact) for the exponent's fixed point.
    __shared__ double s_thi[WP_MAX_CHANNELS][WP_W + 1], s_tlo[WP_MAX_CHANNELS][WP_W + 1];
    __shared__ double s_l2d40[WP_MAX_CHANNELS][WP_W + 1];
    __shared__ float s_thi_f[WP_MAX_CHANNELS][WP_W + 1], s_tlo_f[WP_MAX_CHANNELS][WP_W + 1];
    __shared__ float s_nm[WP_MAX_CHANNELS][WP_W + 1];
    __shared__ int s_ne[WP_MAX_CHANNELS][WP_W + 1];
    if (tabled) {
        for (int k = threadIdx.x; k < C * (WP_W + 1); k += blockDim.x) {
            const int c = k / (WP_W + 1), d = k % (WP_W + 1);
            const double sd = __dmul_rn(dist_cutoff, m.e_sig[c][d]);
            s_thi[c][d] = __dadd_rn(m.e_amu[c][d], sd);
            s_tlo[c][d] = __dsub_rn(m.e_amu[c][d], sd);
            s_thi_f[c][d] = (float)s_thi[c][d];
            s_tlo_f[c][d] = (float)s_tlo[c][d];
            s_l2d40[c][d] = m.e_l2den[c][d] * 0x1p40;
            int ne;
            float nm = (float)frexp(m.e_norm[c][d], &ne);
            if (nm >= 1.0f) {  // rounding up to 1.0
                nm = 0.5f;
                ne += 1;
            }
            s_nm[c][d] = nm;
            s_ne[c][d] = ne;
        }
        __syncthreads();
    }
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
    } else if (tabled) {
        // Without interactions channel c's mu and sigma depend on its own
        // count alone, so the reference's fixed point over the other
        // channels' counts changes nothing here and is skipped; the scans
        // for the first count with mu + s > x and, from there, the first
        // with mu - s > x compare x with the thresholds.
        for (int c = 0; c < C; c++) {
            const double x = rad[t * C + c];
            const float xf = (float)x;
            unsigned cmin = max_num_dyes + 1;
            for (unsigned d = 0; d < max_num_dyes + 1; d++) {
                const float tf = s_thi_f[c][d];
                if (tf > xf || (tf == xf && s_thi[c][d] > x)) {
                    cmin = d;
                    break;
                }
            }
            unsigned cmax = max_num_dyes + 1;
            for (unsigned d = cmin; d < max_num_dyes + 1; d++) {
                const float tf = s_tlo_f[c][d];
                if (tf > xf || (tf == xf && s_tlo[c][d] > x)) {
                    cmax = d;
                    break;
                }
            }
            lo[c] = cmin;
            hi[c] = cmax;
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
                double mu1, s;
                if (tabled) {
                    mu1 = m.e_amu[c][1];
                    s = dist_cutoff * m.e_sig[c][old];
                } else {
                    counts_hi[c] = 1;
                    mu1 = dev_adjusted_mu(m, c, counts_hi);
                    counts_hi[c] = old;
                    double mu = dev_adjusted_mu(m, c, counts_hi);
                    s = dist_cutoff * dev_sigma(m, c, mu);
                }
                // x / 1.0 == x exactly: the division (slow in FP64) only where mu != 1
                const double q = mu1 == 1.0 ? rad[t * C + c] + s : (rad[t * C + c] + s) / mu1;
                unsigned new_cts = (unsigned)lround(q);
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
                double mu, s;
                if (tabled) {
                    mu = m.e_amu[c][d];
                    s = dist_cutoff * m.e_sig[c][d];
                } else {
                    mu = dev_adjusted_mu(m, c, counts_lo);
                    s = dist_cutoff * dev_sigma(m, c, mu);
                }
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
                double mu, s;
                if (tabled) {
                    mu = m.e_amu[c][d];
                    s = dist_cutoff * m.e_sig[c][d];
                } else {
                    mu = dev_adjusted_mu(m, c, counts_hi);
                    s = dist_cutoff * dev_sigma(m, c, mu);
                }
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
                EmitEntry en;
                en.mant = 0.0f;
                en.expo = WP_EXPO_ZERO;
                if ((unsigned)n >= lo[c] && (unsigned)n < hi[c]) {
                    // pdf_helper (channel-model.h:61-70) from the tables:
                    // norm * exp(-offset^2 / den) = norm * 2^y, y in FP64
                    // (as y * 2^40, exact); y rounded to 24 fractional bits
                    // by one conversion to a 64-bit integer gives the
                    // power of two of its integer part exactly and the
                    // fraction exactly as an FP32 number; 2^frac (in
                    // [1, 2)) times norm's mantissa is taken in FP32, which
                    // the FP32 mantissa stored keeps to about one unit in
                    // the last place (FP64 runs at a small fraction of the
                    // FP32 rate on this GPU).  Far tails (y <= -1000, where
                    // FP64 itself nears underflow) take the FP64 exp so
                    // that zeros fall where the reference's do.
                    const double offset = rad[t * C + c] - m.e_amu[c][n];
                    const double y40 = -(offset * offset) * s_l2d40[c][n];
                    if (y40 > -1000.0 * 0x1p40) {
                        // round(y * 2^24): floor(y * 2^40), then to nearest
                        const long long q24 = (__double2ll_rd(y40) + (1ll << 15)) >> 16;
                        const int fl = (int)(q24 >> 24);
                        const float fr = exp2f((float)(int)(q24 & 0xffffff) * 0x1p-24f);
                        const float pm = s_nm[c][n] * fr;  // in [0.5, 2]
                        const bool up = pm >= 1.0f;
                        en.mant = up ? 0.5f * pm : pm;
                        en.expo = s_ne[c][n] + (up ? 1 : 0) + fl;
                        if (en.mant >= 1.0f) {  // rounding up to 1.0
                            en.mant = 0.5f;
                            en.expo += 1;
                        }
                    } else {
                        en = make_entry(m.e_norm[c][n] * exp(-offset * offset / m.e_den[c][n]));
                    }
                }
                out[(t * C + c) * W + n] = en;
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


// One thread per read.
__global__ void wp_read_summary_kernel(BatchArgs a) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.R) return;
    const DevModel& m = *a.model;
    const int T = m.T, C = m.C;
    const uint8_t* lo = a.lo + (long)r * T * C;
    const uint8_t* hi = a.hi + (long)r * T * C;
    uint8_t* Ls = a.Lsuf + (long)r * T * C;
    uint8_t* Up = a.Upre + (long)r * T * C;
    int L[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    for (int t = T - 1; t >= 0; t--)
        for (int c = 0; c < C; c++) {
            L[c] = max(L[c], (int)lo[t * C + c]);
            Ls[t * C + c] = (uint8_t)L[c];
        }
    int U[WP_MAX_CHANNELS] = {255, 255, 255, 255};
    int empty = 0;
    for (int t = 0; t < T; t++) {
        int allow = 1;
        uint32_t lpk = 0, upk = 0;
        for (int c = 0; c < C; c++) {
            U[c] = min(U[c], (int)hi[t * C + c]);
            Up[t * C + c] = (uint8_t)U[c];
            int l = Ls[t * C + c];
            if (l >= U[c]) empty = 1;
            // PeptideEmission::prune_* sets allow_detached =
            // pruned_range.includes_zero() (peptide-emission.cc:198-210).
            if (l != 0 || U[c] == 0) allow = 0;
            lpk |= (uint32_t)l << (8 * c);
            upk |= (uint32_t)U[c] << (8 * c);
        }
        a.allow[(long)r * T + t] = (uint8_t)allow;
        // One word per (read, t) and bound: byte c is channel c.
        a.Lpk[(long)r * T + t] = lpk | ((uint32_t)allow << 31);
        a.Upk[(long)r * T + t] = upk;
    }
    a.flags[r] = (uint8_t)empty;
}

// One thread per (read, t), non-interacting models, after the summary: the
// window-normalised emission factors the engine reads (BatchArgs::gtab, gK,
// gdelta).  For a pair's box [L_t, u) of channel c the engine multiplies the
// window factors by 2^gdelta, which gives exactly mant * 2^(expo - k_box), k_box
// the box's largest exponent (both factors are powers of two and nothing
// leaves the normal range while every factor is within 2^100 of its
// window's largest), and adds sum_c (k_window - gdelta) as the box's
// normalising exponent: the same numbers the engine's own normalisation of
// the box gives.  Where a factor lies further below, gK = WP_GK_NONE and the
// engine normalises that (read, t) itself.
// Shared memory of wp_window_factors_kernel: per item its table row and its
// outputs (C W entries, floats and bytes).
size_t wp_window_smem_bytes(int C, int W, int threads) {
    return (size_t)threads * C * W * (sizeof(EmitEntry) + sizeof(float) + 1);
}

__global__ void wp_window_factors_kernel(BatchArgs a) {
    const DevModel& m = *a.model;
    const int T = m.T, C = m.C, W = a.W;
    const int CW = C * W;
    // The CTA's (read, t) items are consecutive and so are their table rows
    // and output rows (C W entries per item), so the rows go through shared
    // memory: the loads and stores of the CTA are coalesced, not one
    // thread's row after another's.
    extern __shared__ __align__(16) unsigned char w_smem[];
    EmitEntry* s_tab = reinterpret_cast<EmitEntry*>(w_smem);
    float* s_gt = reinterpret_cast<float*>(s_tab + (size_t)blockDim.x * CW);
    uint8_t* s_gd = reinterpret_cast<uint8_t*>(s_gt + (size_t)blockDim.x * CW);
    const long item0 = (long)blockIdx.x * blockDim.x;
    const long n_items_all = (long)a.R * T;
    const int n_items = (int)min((long)blockDim.x, n_items_all - item0);
    const int n_ent = n_items * CW;
    {
        const EmitEntry* src = a.tab + item0 * CW;  // [r][t][c][n]: item (r, t) at (r T + t) C W
        for (int k = threadIdx.x; k < n_ent; k += blockDim.x) s_tab[k] = src[k];
    }
    __syncthreads();
    const long gid = item0 + threadIdx.x;
    if (threadIdx.x < n_items) {
        const int r = (int)(gid / T), t = (int)(gid % T);
        const long rt = (long)r * T + t;
        const EmitEntry* tab = s_tab + threadIdx.x * CW;  // [c W + n]
        float* gt = s_gt + threadIdx.x * CW;
        uint8_t* gd = s_gd + threadIdx.x * CW;
        const uint8_t* lo = a.lo + rt * C;
        const uint8_t* hi = a.hi + rt * C;
        const uint8_t* Ls = a.Lsuf + rt * C;
        const uint8_t* Up = a.Upre + rt * C;
        int K = 0;
        bool ok = true;
        for (int c = 0; c < C; c++) {
            const EmitEntry* row = tab + c * W;
            int km = WP_EXPO_ZERO;  // the window's largest exponent
            for (int n = lo[c]; n < hi[c] && n < W; n++)
                if (row[n].mant != 0.0f) km = max(km, row[n].expo);
            for (int n = 0; n < W; n++) {
                const EmitEntry en = row[n];  // zero outside the window
                float v = 0.0f;
                if (en.mant != 0.0f) {
                    const int d = en.expo - km;
                    if (d < -100)
                        ok = false;
                    else
                        v = en.mant * exp2i(d);
                }
                gt[c * W + n] = v;
            }
            if (km != WP_EXPO_ZERO) K += km;
            // boxes [L_t, u): the window's exponent minus the box's largest (0
            // while the box has no nonzero factor; its pairs get P = 0)
            const int L = Ls[c], U = Up[c];
            int run = WP_EXPO_ZERO;
            for (int u = 1; u <= W; u++) {
                int dl = 0;
                if (u > L && u <= U) {
                    const EmitEntry en = row[u - 1];
                    if (en.mant != 0.0f) run = max(run, en.expo);
                    if (run != WP_EXPO_ZERO) dl = km - run;
                }
                gd[c * W + u - 1] = (uint8_t)(dl <= 100 ? dl : 0);
            }
        }
        a.gK[rt] = ok ? K : WP_GK_NONE;
        if (a.gone) {
            // one-state read box in every channel: the state's own factors
            float mv[3] = {0.0f, 0.0f, 0.0f};
            int K1 = 0;
            bool one = C <= 3;
            for (int c = 0; c < C && one; c++) {
                const int L = Ls[c];
                if (Up[c] != L + 1 || L >= W) {
                    one = false;
                    break;
                }
                const EmitEntry en = tab[c * W + L];
                mv[c] = en.mant;
                if (en.mant != 0.0f) K1 += en.expo;
            }
            a.gone[rt] = make_float4(mv[0], mv[1], mv[2], __int_as_float(one ? K1 : WP_GK_NONE));
        }
    }
    __syncthreads();
    float* dst_gt = a.gtab + item0 * CW;
    uint8_t* dst_gd = a.gdelta + item0 * CW;
    for (int k = threadIdx.x; k < n_ent; k += blockDim.x) {
        dst_gt[k] = s_gt[k];
        dst_gd[k] = s_gd[k];
    }
}

// One CTA per read (at most 1,024 threads, a multiple of 32).  CTA-aggregated
// appends keep the read's pairs of each list contiguous (they share the
// read's data in L1) and cost one global atomic per list per 2,048 slots.
__global__ void wp_compact_kernel(BatchArgs a) {
    const int r = blockIdx.x;
    const DevModel& m = *a.model;
    const int C = m.C;
    const int g0 = slot_begin(a, r);
    const int g1 = a.slot_off ? a.slot_off[r + 1] : g0 + a.P;
    const bool read_empty = a.flags[r] != 0;
    int minD[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    for (int c = 0; c < C; c++) minD[c] = a.Lsuf[(long)r * m.T * C + c];  // L_0
    const int lane = threadIdx.x & 31;
    // the read's box words, shared by all its pairs
    __shared__ uint32_t sL[WP_MAX_TIMESTEPS], sU[WP_MAX_TIMESTEPS];
    __shared__ int s_live;  // the read's non-empty pairs
    if (threadIdx.x == 0) s_live = 0;
    for (int t = threadIdx.x; t < m.T; t += blockDim.x) {
        sL[t] = a.Lpk[(long)r * m.T + t];
        sU[t] = a.Upk[(long)r * m.T + t];
    }
    __syncthreads();
    // The largest box of this read's pairs per distinct dye-count vector
    // (pair_vmax depends on the peptide through its dye counts only).
    __shared__ int s_vmax[WP_COMPACT_UNIQ];
    const bool vtab = a.uniq_D && a.n_uniq > 0 && a.n_uniq <= WP_COMPACT_UNIQ && !read_empty;
    if (vtab) {
        for (int u = threadIdx.x; u < a.n_uniq; u += blockDim.x) {
            const uint32_t Dw = a.uniq_D[u];
            bool ok = true;
            for (int c = 0; c < C; c++)
                if ((int)((Dw >> (8 * c)) & 0xffu) < minD[c]) ok = false;
            s_vmax[u] = ok ? pair_vmax_w(C, m.T, sL, sU, Dw) : 0;
        }
    }
    // Candidate mode: the read's slots in the peptides' shape order (up to
    // WP_COMPACT_SORT slots; more keep their order), sorted here by a
    // bitonic sort of (shape rank, slot) keys.
    __shared__ unsigned long long order[WP_COMPACT_SORT];
    const int ns = g1 - g0;
    const bool sorted = a.cand && a.shape_rank && ns <= WP_COMPACT_SORT;
    if (sorted) {
        int n2 = 1;
        while (n2 < ns) n2 <<= 1;
        for (int i = threadIdx.x; i < n2; i += blockDim.x)
            order[i] = i < ns ? ((unsigned long long)(unsigned)a.shape_rank[a.cand[g0 + i]] << 32) | (unsigned)i
                              : ~0ull;
        __syncthreads();
        for (int size = 2; size <= n2; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const bool up = (i & size) == 0;
                        const unsigned long long x = order[i], y = order[j];
                        if ((x > y) == up) {
                            order[i] = y;
                            order[j] = x;
                        }
                    }
                }
                __syncthreads();
            }
    }
    __syncthreads();
    // Lists are appended per CTA: the read's pairs of a list take one
    // contiguous range (one global atomic per list per chunk of slots, not
    // one per warp), in the walk's order.
    constexpr int NL = WP_MAX_TIERS + 1;
    __shared__ uint8_t s_dest[WP_COMPACT_CHUNK];
    __shared__ int s_off[WP_COMPACT_CHUNK / 32][NL];  // per (iteration, warp): count, then start
    const int wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int per_chunk = (WP_COMPACT_CHUNK / blockDim.x) * blockDim.x;
    for (int c0 = g0; c0 < g1; c0 += per_chunk) {
        const int c1 = min(g1, c0 + per_chunk);
        const int nit = (c1 - c0 + blockDim.x - 1) / blockDim.x;
        // phase A: each slot's list (or none), counted per warp and list
        for (int it = 0; it < nit; it++) {
            const int base = c0 + it * blockDim.x;
            // Walk the peptides in shape order (all-peptides mode: the
            // global order; candidate mode: the read's sorted slots), so
            // that the engine's warps get pairs of similar size; results
            // still go to their own slots, so the candidate order (ties) is
            // unchanged.
            int g = base + threadIdx.x;
            if (g < g1 && a.perm) g = g0 + a.perm[g - g0];
            if (g < g1 && sorted) g = g0 + (int)(order[g - g0] & 0xffffffffu);
            int dest = -1;  // tier index, WP_MAX_TIERS: the dense kernel's list
            if (base + threadIdx.x < g1) {
                int p = slot_pep(a, r, g);
                const PeptideRec& pep = a.peps[p];
                bool live = !read_empty;
                for (int c = 0; c < C; c++)
                    if (pep.D[c] < minD[c]) live = false;
                if (live) {
                    // the pair's largest box waits in its result slot for
                    // the engine, which checks it against its slab before
                    // any write
                    const int vm = vtab ? s_vmax[a.pep_u[p]]
                                        : pair_vmax_w(C, m.T, sL, sU,
                                                      (uint32_t)pep.D[0] | ((uint32_t)pep.D[1] << 8) |
                                                              ((uint32_t)pep.D[2] << 16) | ((uint32_t)pep.D[3] << 24));
                    a.res_expo[g] = vm;
                    dest = 0;
                    if (a.n_tiers > 0) {
                        dest = WP_MAX_TIERS;
                        for (int k = a.n_tiers - 1; k >= 0; k--)
                            if (vm <= a.tier_half[k]) dest = k;
                        if (dest == WP_MAX_TIERS && !a.route_dense) {
                            atomicExch(a.err, 2);  // no shape holds this pair
                            dest = -1;
                        }
                    }
                }
                if (dest < 0) {
                    a.res_mant[g] = 0.0f;
                    a.res_expo[g] = 0;
                }
            }
            s_dest[it * blockDim.x + threadIdx.x] = dest < 0 ? 0xffu : (uint8_t)dest;
            const unsigned lm = __ballot_sync(0xffffffffu, dest >= 0);
            if (lane == 0 && lm) atomicAdd(&s_live, __popc(lm));
            for (int k = 0; k < NL; k++) {
                const unsigned mask = __ballot_sync(0xffffffffu, dest == k);
                if (lane == 0) s_off[it * nwarp + wid][k] = __popc(mask);
            }
        }
        __syncthreads();
        // one range per list: its start, then each (iteration, warp)'s start
        if (threadIdx.x < NL) {
            const int k = threadIdx.x;
            const int n = nit * nwarp;
            int total = 0;
            for (int i = 0; i < n; i++) total += s_off[i][k];
            int start = 0;
            if (total > 0) {
                const bool dense = k == WP_MAX_TIERS;
                int* count = dense ? a.ovf_count : a.n_tiers > 0 ? a.tier_count[k] : a.work_count;
                start = atomicAdd(count, total);
            }
            for (int i = 0; i < n; i++) {
                const int c = s_off[i][k];
                s_off[i][k] = start;
                start += c;
            }
        }
        __syncthreads();
        // phase B: the appends
        for (int it = 0; it < nit; it++) {
            const int base = c0 + it * blockDim.x;
            int g = base + threadIdx.x;
            if (g < g1 && a.perm) g = g0 + a.perm[g - g0];
            if (g < g1 && sorted) g = g0 + (int)(order[g - g0] & 0xffffffffu);
            const uint8_t d8 = s_dest[it * blockDim.x + threadIdx.x];
            const int dest = d8 == 0xffu ? -1 : (int)d8;
            for (int k = 0; k < NL; k++) {
                const unsigned mask = __ballot_sync(0xffffffffu, dest == k);
                if (dest == k) {
                    const bool dense = k == WP_MAX_TIERS;
                    int2* list = dense ? a.ovf : a.n_tiers > 0 ? a.tier_list[k] : a.work;
                    list[s_off[it * nwarp + wid][k] + __popc(mask & ((1u << lane) - 1))] = make_int2(r, g);
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && a.live_count && s_live) atomicAdd(a.live_count, s_live);
}

// All-peptides mode, one warp per read: the compaction of wp_compact_kernel
// done once per group of peptides sharing a dye-count vector (a run of the
// shape order).  Whether a pair is empty (L_0 > D on some channel) and its
// largest box depend on the peptide through that vector alone, so each group
// is routed as a whole: its pairs go, in the shape order, to the list of the
// first engine pass whose slab holds the box.  Result indices are dense
// (BatchArgs::pair_info): the read's non-empty pairs take one contiguous
// range in the order of the appends, each with its peptide and box size
// beside it, so the engine's result writes and the reduce's reads are
// coalesced and empty pairs cost nothing (P = 0 without a result).  The
// read's pairs of a list take one contiguous range (one global atomic per
// list).
// Persistent CTAs (wp_compact_groups_smem_bytes): the groups and the shape
// order are staged in shared memory once per CTA, so a warp's per-read work
// waits on global memory only for the read's box words and the list atomics.
size_t wp_compact_groups_smem_bytes(int n_grp, int P) {
    size_t b = (size_t)(n_grp + 1) * sizeof(int) + (size_t)n_grp * sizeof(uint32_t);
    b += (size_t)WP_GROUP_WARPS * n_grp * (sizeof(uint32_t) + sizeof(uint16_t));  // sort keys, order
    b = (b + 15) & ~(size_t)15;
    if (P <= WP_GROUP_PERM_SMEM) b += (size_t)P * sizeof(int);
    return (b + 15) & ~(size_t)15;
}

__global__ void __launch_bounds__(WP_GROUP_WARPS * 32) wp_compact_groups_kernel(BatchArgs a) {
    constexpr int NL = WP_MAX_TIERS + 1;
    extern __shared__ __align__(16) unsigned char g_smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ uint32_t sL[WP_GROUP_WARPS][WP_MAX_TIMESTEPS], sU[WP_GROUP_WARPS][WP_MAX_TIMESTEPS];
    __shared__ uint16_t s_live[WP_GROUP_WARPS][WP_GROUP_MAX];  // routed groups, in order
    __shared__ uint16_t s_vm[WP_GROUP_WARPS][WP_GROUP_MAX];    // per group: largest box (engine passes)
    __shared__ uint8_t s_dest[WP_GROUP_WARPS][WP_GROUP_MAX];   // per group: list (WP_MAX_TIERS: dense)
    __shared__ uint16_t s_bkt[WP_GROUP_WARPS][WP_GROUP_BUCKETS];  // the counting sort's buckets
    const int n_grp = a.n_grp;
    int* gstart = reinterpret_cast<int*>(g_smem);
    uint32_t* gD = reinterpret_cast<uint32_t*>(gstart + n_grp + 1);
    const bool perm_smem = a.P <= WP_GROUP_PERM_SMEM;
    uint32_t* s_key = gD + n_grp + (size_t)wid * n_grp;  // this warp's sort keys
    uint16_t* s_ord = reinterpret_cast<uint16_t*>(gD + n_grp + (size_t)WP_GROUP_WARPS * n_grp) + (size_t)wid * n_grp;
    int* sperm = reinterpret_cast<int*>(
            (reinterpret_cast<uintptr_t>(gD + n_grp + (size_t)WP_GROUP_WARPS * n_grp) +
             (size_t)WP_GROUP_WARPS * n_grp * sizeof(uint16_t) + 15) & ~(uintptr_t)15);
    for (int i = threadIdx.x; i <= n_grp; i += blockDim.x) gstart[i] = a.grp_start[i];
    for (int i = threadIdx.x; i < n_grp; i += blockDim.x) gD[i] = a.grp_D[i];
    if (perm_smem)
        for (int i = threadIdx.x; i < a.P; i += blockDim.x) sperm[i] = a.perm[i];
    __syncthreads();
    const int* perm = perm_smem ? sperm : a.perm;
    const DevModel& m = *a.model;
    const int T = m.T, C = m.C;
    const int nwarps = gridDim.x * WP_GROUP_WARPS;
    for (int r = blockIdx.x * WP_GROUP_WARPS + wid; r < a.R; r += nwarps) {
        for (int t = lane; t < T; t += 32) {
            sL[wid][t] = a.Lpk[(long)r * T + t];
            sU[wid][t] = a.Upk[(long)r * T + t];
        }
        const bool read_empty = a.flags[r] != 0;
        __syncwarp();
        const uint32_t L0 = sL[wid][0] & 0x7f7f7f7fu;
        // U_max - 1 per channel (byte): a group's dyes clamped to it give
        // the same boxes at every timestep (min(U_t, D + 1) = min(U_t,
        // D' + 1) for D' = min(D, U_max - 1)), so pairs whose clamped counts
        // agree run the same steps; the appends order groups by them
        uint32_t um = 0;
        for (int t = lane; t < T; t += 32) um = __vmaxu4(um, sU[wid][t]);
        for (int o = 16; o > 0; o >>= 1) um = __vmaxu4(um, __shfl_xor_sync(0xffffffffu, um, o));
        const uint32_t um1 = __vsubus4(um, 0x01010101u);  // U >= 1 on every channel of a read with pairs
        // the non-empty groups (every byte D_c >= L_0,c: bytes below 128,
        // bit 7 of (D | 0x80..) - L0 stays set exactly where D_c >= L_0,c;
        // bytes past the channels are 0), keyed by their clamped counts
        int n_live = 0;  // warp-uniform
        for (int u0 = 0; u0 < n_grp && !read_empty; u0 += 32) {
            const int u = u0 + lane;
            bool live = false;
            uint32_t D = 0;
            if (u < n_grp) {
                D = gD[u];
                live = ((((D | 0x80808080u) - L0) & 0x80808080u) == 0x80808080u);
            }
            const unsigned lm = __ballot_sync(0xffffffffu, live);
            if (live) {
                const int at = n_live + __popc(lm & ((1u << lane) - 1));
                s_live[wid][at] = (uint16_t)u;
                // sort key: clamped counts (4 bits a channel), position
                const uint32_t dc = __vminu4(D, um1);
                const uint32_t d16 = (dc & 0xfu) | ((dc >> 4) & 0xf0u) | ((dc >> 8) & 0xf00u) | ((dc >> 12) & 0xf000u);
                s_key[at] = (d16 << 9) | (uint32_t)at;
            }
            n_live += __popc(lm);
        }
        __syncwarp();
        // The groups in key order (s_ord).  When the clamped counts take at
        // most WP_GROUP_BUCKETS values: a stable counting sort over them as
        // a mixed-radix number, channel C - 1 most significant (the order
        // of the key's bits), 32 positions a round with one writer per
        // bucket and round; else the rank of each key among all (keys are
        // distinct).  Both give the same order.
        int range = 1;
        for (int c = 0; c < C; c++) range *= min((int)((um1 >> (8 * c)) & 0xffu), 15) + 1;
        if (range <= WP_GROUP_BUCKETS) {
            uint16_t* bk = s_bkt[wid];
            auto bucket = [&](int i) {
                const uint32_t d16 = s_key[i] >> 9;
                int b = 0;
                for (int c = C - 1; c >= 0; c--)
                    b = b * (min((int)((um1 >> (8 * c)) & 0xffu), 15) + 1) + (int)((d16 >> (4 * c)) & 0xfu);
                return b;
            };
            for (int b = lane; b < range; b += 32) bk[b] = 0;
            __syncwarp();
            for (int i0 = 0; i0 < n_live; i0 += 32) {
                const int i = i0 + lane;
                const int b = i < n_live ? bucket(i) : -1 - lane;  // idle lanes: a bucket of their own
                const unsigned peers = __match_any_sync(0xffffffffu, b);
                if (i < n_live && lane == __ffs(peers) - 1) bk[b] = (uint16_t)(bk[b] + __popc(peers));
                __syncwarp();
            }
            // bucket sizes to first positions: each lane scans a block of buckets
            const int per = (range + 31) >> 5;
            const int b0 = min(lane * per, range), b1 = min(b0 + per, range);
            int sz = 0;
            for (int b = b0; b < b1; b++) sz += bk[b];
            int incl = sz;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            int run = incl - sz;
            for (int b = b0; b < b1; b++) {
                const int n = bk[b];
                bk[b] = (uint16_t)run;
                run += n;
            }
            __syncwarp();
            for (int i0 = 0; i0 < n_live; i0 += 32) {
                const int i = i0 + lane;
                const int b = i < n_live ? bucket(i) : -1 - lane;
                const unsigned peers = __match_any_sync(0xffffffffu, b);
                if (i < n_live) s_ord[bk[b] + __popc(peers & ((1u << lane) - 1))] = (uint16_t)i;
                __syncwarp();
                if (i < n_live && lane == __ffs(peers) - 1) bk[b] = (uint16_t)(bk[b] + __popc(peers));
                __syncwarp();
            }
        } else {
            for (int i = lane; i < n_live; i += 32) {
                const uint32_t ki = s_key[i];
                int rank = 0;
                for (int j = 0; j < n_live; j++) rank += s_key[j] < ki ? 1 : 0;
                s_ord[rank] = (uint16_t)i;
            }
        }
        __syncwarp();
        // The largest box depends on the counts through the clamped ones
        // alone (pair_vmax takes min(U_t, D + 1) = min(U_t, D' + 1)), so it
        // is computed once per run of equal clamped counts in key order:
        // the runs' clamped counts are listed first (in the sort's buckets,
        // free now), then the lanes take one run each, and the pass list of
        // every group follows from its run's box.
        uint16_t* runs = s_bkt[wid];
        int n_runs = 0;  // warp-uniform
        for (int o0 = 0; o0 < n_live; o0 += 32) {
            const int o = o0 + lane;
            bool start = false;
            uint32_t dk = 0;
            if (o < n_live) {
                dk = s_key[s_ord[o]] >> 9;
                start = o == 0 || (s_key[s_ord[o - 1]] >> 9) != dk;
            }
            const unsigned sm = __ballot_sync(0xffffffffu, start);
            if (start) runs[n_runs + __popc(sm & ((1u << lane) - 1))] = (uint16_t)dk;
            n_runs += __popc(sm);
        }
        __syncwarp();
        for (int k0 = 0; k0 < n_runs; k0 += 32) {
            const int k = k0 + lane;
            int vm = 0;
            if (k < n_runs) {
                const uint32_t dk = runs[k];
                const uint32_t Dw = (dk & 0xfu) | ((dk & 0xf0u) << 4) | ((dk & 0xf00u) << 8) | ((dk & 0xf000u) << 12);
                vm = pair_vmax_w(C, T, sL[wid], sU[wid], Dw);
            }
            __syncwarp();
            if (k < n_runs) runs[k] = (uint16_t)min(vm, 65535);  // above every slab half
        }
        __syncwarp();
        int tot[NL];
#pragma unroll
        for (int k = 0; k < NL; k++) tot[k] = 0;
        int run0 = 0;  // runs started before this chunk (warp-uniform)
        for (int o0 = 0; o0 < n_live; o0 += 32) {
            const int o = o0 + lane;
            int i = 0;
            bool start = false;
            if (o < n_live) {
                i = s_ord[o];
                start = o == 0 || (s_key[s_ord[o - 1]] >> 9) != (s_key[i] >> 9);
            }
            const unsigned sm = __ballot_sync(0xffffffffu, start);
            if (o < n_live) {
                const int v = runs[run0 + __popc(sm & (0xffffffffu >> (31 - lane))) - 1];
                const int u = s_live[wid][i];
                int dest = 0;  // -2: no shape holds these pairs (P = 0, err = 2)
                if (a.n_tiers > 0) {
                    dest = WP_MAX_TIERS;
                    for (int k = a.n_tiers - 1; k >= 0; k--)
                        if (v <= a.tier_half[k]) dest = k;
                    if (dest == WP_MAX_TIERS && !a.route_dense) dest = -2;
                }
                if (dest == -2) atomicExch(a.err, 2);
                s_vm[wid][i] = (uint16_t)v;
                s_dest[wid][i] = (uint8_t)(dest < 0 ? 0xffu : dest);
                const int cnt = gstart[u + 1] - gstart[u];
#pragma unroll
                for (int k = 0; k < NL; k++)
                    if (dest == k) tot[k] += cnt;
            }
            run0 += __popc(sm);
        }
        // each list's range for this read: lane k takes list k's atomic
        int base[NL];
        int mine = 0, live_pairs = 0;
#pragma unroll
        for (int k = 0; k < NL; k++) {
            int v = tot[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            live_pairs += v;
            if (lane == k) mine = v;
        }
        // and lane NL the read's range of result indices (the count of
        // non-empty pairs is the allocator)
        int b = 0;
        if (lane < NL && mine > 0) {
            int* count = lane == WP_MAX_TIERS ? a.ovf_count : a.n_tiers > 0 ? a.tier_count[lane] : a.work_count;
            b = atomicAdd(count, mine);
        } else if (lane == NL && live_pairs > 0) {
            b = atomicAdd(a.live_count, live_pairs);
        }
#pragma unroll
        for (int k = 0; k < NL; k++) base[k] = __shfl_sync(0xffffffffu, b, k);
        int dpos = __shfl_sync(0xffffffffu, b, NL);
        if (lane == 0) {
            a.rd_base[r] = dpos;
            a.rd_n[r] = live_pairs;
        }
        __syncwarp();
        // The appends, in key order, 32 groups a round: a group's pairs
        // take the next places of its list and the next result indices
        // (scans of the group sizes, per list and over all), and the lanes
        // share the round's pairs.  Groups no pass holds (err = 2) take
        // neither: P = 0.
        for (int o0 = 0; o0 < n_live; o0 += 32) {
            const int o = o0 + lane;
            int cnt = 0, p0 = 0, vm = 0, d8 = 0xff;
            if (o < n_live) {
                const int i = s_ord[o];
                d8 = s_dest[wid][i];
                if (d8 != 0xff) {
                    const int u = s_live[wid][i];
                    p0 = gstart[u];
                    cnt = gstart[u + 1] - p0;
                    vm = s_vm[wid][i];
                }
            }
            int lpos = 0;  // the group's first place in its list
#pragma unroll
            for (int k = 0; k < NL; k++) {
                const int v = d8 == k ? cnt : 0;
                int inc = v;
                for (int sft = 1; sft < 32; sft <<= 1) {
                    const int w = __shfl_up_sync(0xffffffffu, inc, sft);
                    if (lane >= sft) inc += w;
                }
                if (d8 == k) lpos = base[k] + inc - v;
                base[k] += __shfl_sync(0xffffffffu, inc, 31);
            }
            int incl = cnt;
            for (int sft = 1; sft < 32; sft <<= 1) {
                const int w = __shfl_up_sync(0xffffffffu, incl, sft);
                if (lane >= sft) incl += w;
            }
            const int excl = incl - cnt;  // the group's first pair in the round
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int q0 = 0; q0 < total; q0 += 32) {
                const int q = q0 + lane;
                // the group holding pair q: the last lane whose first pair is <= q
                int src = 0;
                for (int sft = 16; sft > 0; sft >>= 1) {
                    const int e = __shfl_sync(0xffffffffu, excl, src + sft);
                    if (e <= q) src += sft;
                }
                const int g_excl = __shfl_sync(0xffffffffu, excl, src);
                const int g_p0 = __shfl_sync(0xffffffffu, p0, src);
                const int g_vm = __shfl_sync(0xffffffffu, vm, src);
                const int g_lpos = __shfl_sync(0xffffffffu, lpos, src);
                const int g_d8 = __shfl_sync(0xffffffffu, d8, src);
                if (q < total) {
                    const int j = q - g_excl;
                    const int d = dpos + q;
                    int2* list = a.work;
#pragma unroll
                    for (int k = 0; k < NL; k++)
                        if (g_d8 == k) list = k == WP_MAX_TIERS ? a.ovf : a.n_tiers > 0 ? a.tier_list[k] : a.work;
                    a.pair_info[d] = make_int2(perm[g_p0 + j], g_vm);  // slot offset = peptide
                    list[g_lpos + j] = make_int2(r, d);
                }
            }
            dpos += total;
        }
        __syncwarp();
    }
}
