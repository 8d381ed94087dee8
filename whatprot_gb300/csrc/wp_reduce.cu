// wp_reduce.cu -- per-read reductions over the per-pair probabilities, the
// visited-work counter and the FP32 throughput probe.
//
//   wp_reduce_kernel        one warp per read: HMMClassifier::classify_helper
//                           (classifiers/hmm-classifier.h:45-78) -- the best
//                           peptide (strict '>', so the first candidate wins
//                           ties), its probability, the total weighted by
//                           peptide multiplicity, and the NaN patch
//                           (:73-76).  Deterministic: fixed lane assignment
//                           and a fixed butterfly.
//   wp_logp_kernel          log P per slot.
//   wp_count_flops_kernel   the pruned schedule's visited-state op count.
//   wp_fma_probe_kernel     FP32 FMA throughput.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

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


// Exact FP32 sum of two floats as (s, err): s + err == a + b (Knuth's
// TwoSum, six additions, no branch).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
    s = a + b;
    const float bp = s - a;
    const float ap = s - bp;
    err = (a - ap) + (b - bp);
}

// One warp per read (blockDim.x == 128: four reads per CTA), one pass over
// the read's slots.  Each lane keeps its best candidate and the sum of its
// slots' P * count relative to 2^El, El the largest exponent it has met (the
// sum is rescaled by an exact power of two when El grows).  The sum is a
// float pair (hi, lo) fed by exact products (mant * count and its FMA
// remainder) through TwoSum, about 48 significant bits, so the per-slot work
// stays on the FP32 pipes: this GPU's FP64 rate is a small fraction of its
// FP32 rate and an FP64 multiply-add per slot made this kernel FP64-bound.
// Terms below 2^-100 of the lane's reference are dropped (below the FP64
// resolution of a total that holds at least one term of 2^El / 2).  Counts
// of 2^24 or more (not exact in FP32) are added as two terms.  The lanes'
// sums meet in FP32 pairs relative to E, the best's exponent.
__global__ void wp_reduce_kernel(BatchArgs a, int32_t* __restrict__ out_id,
                                 double* __restrict__ out_score, double* __restrict__ out_total,
                                 double* __restrict__ out_log, const int* __restrict__ pep_ids) {
    const int r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (r >= a.R) return;
    const int g0 = slot_begin(a, r);
    const int g1 = a.slot_off ? a.slot_off[r + 1] : g0 + a.P;
    Cand best = {0.0f, 0, INT_MAX, -1};
    // Result indices i0 .. i1 - 1: the read's slots, or (pair_info) its
    // non-empty pairs, each with its slot offset beside it.  A pair without
    // a result index has P = 0, and as the first slot wins among zeros, the
    // first slot stands for all of them.
    const bool dense = a.pair_info != nullptr;
    int i0 = g0, i1 = g1;
    if (dense) {
        i0 = i1 = 0;
        if (g1 > g0) {
            i0 = a.rd_base[r];
            i1 = i0 + a.rd_n[r];
            best.mant = 0.0f;
            best.expo = 0;
            best.key = 0;
            best.idx = g0;
        }
    }
    int El = INT_MIN;  // the lane's reference exponent (none yet)
    float hi = 0.0f, lo = 0.0f;
    // adds mm * cf * s2 (cf an integer exact in FP32, s2 a power of two):
    // the product exactly as its FP32 rounding and the FMA remainder
    auto add_term = [&](float mm, float cf, float s2) {
        const float p = mm * cf;
        const float pe = fmaf(mm, cf, -p);  // exact: p + pe == mm * cf
        float sum, err;
        two_sum(hi, p * s2, sum, err);
        hi = sum;
        lo += err + pe * s2;
    };
    // four results per lane in flight: the loads first, then the results
    // in the lane's order (i, i + 32, i + 64, ...)
    for (int ib = i0 + lane; ib < i1; ib += 128) {
        float mv[4];
        int ev[4], cv[4], kv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = ib + 32 * u;
            mv[u] = 0.0f;
            ev[u] = 0;
            cv[u] = 0;
            kv[u] = 0;
            if (i < i1) {
                const int key = dense ? a.pair_info[i].x : i - g0;  // slot offset
                mv[u] = a.res_mant[i];
                ev[u] = a.res_expo[i];
                cv[u] = a.counts[slot_pep(a, r, g0 + key)];
                kv[u] = key;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (ib + 32 * u >= i1) break;
            const float mm = mv[u];
            const int ex = ev[u];
            Cand c = {mm, ex, kv[u], g0 + kv[u]};
            if (cand_better(c, best)) best = c;
            if (mm > 0.0f) {
                if (ex > El) {
                    const float f = El == INT_MIN || El - ex < -100 ? 0.0f : exp2i(El - ex);
                    hi *= f;
                    lo *= f;
                    El = ex;
                }
                const int d = ex - El;
                if (d >= -100) {
                    const int cnt = cv[u];
                    const float s2 = exp2i(d);
                    if (cnt < (1 << 24)) {
                        add_term(mm, (float)cnt, s2);
                    } else {  // not exact in FP32: its high and low bits apart
                        add_term(mm, (float)(cnt & ~0xfff), s2);
                        add_term(mm, (float)(cnt & 0xfff), s2);
                    }
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        Cand c;
        c.mant = __shfl_xor_sync(0xffffffffu, best.mant, o);
        c.expo = __shfl_xor_sync(0xffffffffu, best.expo, o);
        c.key = __shfl_xor_sync(0xffffffffu, best.key, o);
        c.idx = __shfl_xor_sync(0xffffffffu, best.idx, o);
        if (cand_better(c, best)) best = c;
    }
    // E: the best's exponent, the largest exponent of any nonzero slot
    // (El <= E on every lane).  The lanes' pairs meet relative to 2^E in
    // FP32: scaled by 2^(El - E) (exact, or so far below the best's own
    // term, 2^(E - 1) or more, that FP64 would not hold them either), then
    // summed over the warp with TwoSum, the errors kept in the low words;
    // FP64 (a slow pipe on this GPU) only for lane 0's final sum.
    const int E = best.mant > 0.0f ? best.expo : 0;
    float th = 0.0f, tl = 0.0f;
    if (El != INT_MIN) {
        const float sf = exp2i(max(El - E, -200));
        th = hi * sf;
        tl = lo * sf;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, th, o);
        const float ol = __shfl_xor_sync(0xffffffffu, tl, o);
        float sum, err;
        two_sum(th, oh, sum, err);
        th = sum;
        tl = (tl + ol) + err;
    }
    if (lane != 0) return;
    const double tot = (double)th + (double)tl;
    if (best.idx < 0) {  // no candidates
        out_id[r] = -1;
        out_score[r] = 0.0;
        out_total[r] = 1.0;
        if (out_log) out_log[r] = -INFINITY;
        return;
    }
    out_id[r] = pep_ids[slot_pep(a, r, best.idx)];
    const double sc = (double)best.mant;
    // the reference's NaN patch (score / total NaN): with sc in [0, 1) that
    // is the case exactly when tot is not positive (or NaN)
    if (!(tot > 0.0)) {
        out_score[r] = 0.0;
        out_total[r] = 1.0;
        if (out_log) out_log[r] = -INFINITY;
        return;
    }
    // sc * 2^E and tot * 2^E; where both stay normal that is an add to
    // their exponent fields (sc, tot > 0), else ldexp
    const long long sb = __double_as_longlong(sc), tb = __double_as_longlong(tot);
    const int es = (int)(sb >> 52) + E, et = (int)(tb >> 52) + E;
    if (sb > 0 && es >= 1 && es <= 2046 && et >= 1 && et <= 2046) {
        out_score[r] = __longlong_as_double(sb + ((long long)E << 52));
        out_total[r] = __longlong_as_double(tb + ((long long)E << 52));
    } else {
        const double s_abs = ldexp(sc, E), t_abs = ldexp(tot, E);
        if (s_abs >= DBL_MIN && isfinite(s_abs) && isfinite(t_abs)) {
            out_score[r] = s_abs;
            out_total[r] = t_abs;
        } else {  // outside the double range: same power of two on both
            out_score[r] = sc;
            out_total[r] = tot;
        }
    }
    if (out_log) out_log[r] = log(sc) + (double)E * 0.69314718055994530942;
}

// log P per slot (-inf where P == 0).
__global__ void wp_logp_kernel(const float* __restrict__ mant, const int* __restrict__ expo, long n,
                               double* __restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float mm = mant[i];
    out[i] = mm > 0.0f ? log((double)mm) + (double)expo[i] * 0.69314718055994530942 : -INFINITY;
}

// ---------------------------------------------------------------- flops --

// Visited-state operation count of the reference's pruned schedule for one
// pair, from the closed-form boxes (see the header comment).  One thread per
// (read, peptide).  Sums per read into out[r] (exact: integers < 2^53).
__global__ void wp_count_flops_kernel(BatchArgs a, double* __restrict__ out) {
    const DevModel& m = *a.model;
    const int T = m.T, C = m.C;
    long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)a.R * a.P) return;
    int r = (int)(gid / a.P), p = (int)(gid % a.P);
    const uint8_t* lo = a.lo + (long)r * T * C;
    const uint8_t* hi = a.hi + (long)r * T * C;
    const PeptideRec& pep = a.peps[p];
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
