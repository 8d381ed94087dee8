// wp_nn.cu -- the kNN stage of NNClassifier / HybridClassifier
// (classifiers/nn-classifier.cc:120-215, kd-tree/*) on the GPU.
//
// The reference searches a kd-tree for the entries (unique dye-tracks) whose
// simulated hits add up to k, weights each by exp(-d^2 / 2 sig^2) and scores
// every source peptide id.  Here the search is brute force, as a tiled FP32
// contraction of queries against all entries, in four kernels:
//
//   wp_nn_estimate_kernel distances to a sample of the entries place each
//                         query's distance bins around its k-hit radius
//   wp_nn_hist_kernel     every (query, entry) squared distance, binned on a
//                         log scale (16 bins per octave); per query a histogram
//                         of hits per bin gives the bin b* where the running
//                         hits reach k, the hits below it and an upper bound
//                         on the entries at or below it.
//   wp_nn_collect_kernel  the same distances again; each query (one thread)
//                         appends the entries in bins <= b* to its candidate
//                         list, in entry order (deterministic).
//   wp_nn_select_kernel   one warp per query: the exact k-hit set (entries in
//                         bins < b*, then those of bin b* by a hits-weighted
//                         radix select on the distance bits, ties by entry
//                         index), the weighted scores per peptide (per-id sums
//                         formed in a fixed order), the total, and the top h
//                         ids in ascending (score, id) order.
//
// The set is the shortest prefix of the entries sorted by (squared
// distance, entry index) whose hits reach k: what KBest (k-best.h:26-42)
// holds when entries arrive nearest first.  The kd-tree's visiting order can
// leave a few more far entries in the reference's set.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cub/cub.cuh>

#include "wp_common.cuh"

#define NN_NB 64           // distance bins per query
#define NN_TE 32           // entries per shared-memory tile
#define NN_THREADS 256     // threads per CTA in the distance kernels
#define NN_QPT 1           // queries per thread (one: a warp's 32 sorted reads share
                           // fewer far tiles than 64 would)
#define NN_QPB (NN_THREADS * NN_QPT)
#define NN_SEL_WARPS 4     // warps per CTA in the select kernel
#define NN_HMAX 1024       // largest h

// Coarse log-scale bin of a squared distance, for the estimate: bin 1
// starts at 2^-6, four bins per octave (the exponent and the top two
// mantissa bits of the float), bin 0 below, bin NB-1 open-ended.
__device__ __forceinline__ int nn_coarse_bin(float d2) {
    const int b = (int)(__float_as_uint(d2) >> 21) - ((127 - 6) << 2) + 1;
    return b < 0 ? 0 : (b > NN_NB - 1 ? NN_NB - 1 : b);
}

// Fine bin of a squared distance for one query: sixteen bins per octave
// (exponent and top four mantissa bits), bin 1 starting at the query's
// origin `base` (in units of float bits >> 19), bin 0 below, bin NB-1
// open-ended: 62 fine bins span almost four octaves around the query's
// estimated k-hit radius.  Monotone in d2.
__device__ __forceinline__ int nn_bin(float d2, int base) {
    const int b = (int)(__float_as_uint(d2) >> 19) - base + 1;
    return b < 0 ? 0 : (b > NN_NB - 1 ? NN_NB - 1 : b);
}

// Squared distance of a query (registers) to an entry (shared memory); the
// same code in both distance kernels, so both see the same float.
template <int DP>
__device__ __forceinline__ float nn_d2(const float* q, const float* e) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 4) {
        const float4 v = *reinterpret_cast<const float4*>(e + i);
        const float x0 = q[i] - v.x, x1 = q[i + 1] - v.y, x2 = q[i + 2] - v.z, x3 = q[i + 3] - v.w;
        a0 = fmaf(x0, x0, a0);
        a1 = fmaf(x1, x1, a1);
        a2 = fmaf(x2, x2, a2);
        a3 = fmaf(x3, x3, a3);
    }
    return (a0 + a1) + (a2 + a3);
}


// Squared distance for binning, as |q|^2 + |e|^2 - 2 q.e: one multiply-add
// per coordinate instead of a subtract and a multiply-add.  Its rounding
// error (about 1e-7 of |q|^2 + |e|^2) only moves entries lying that close to
// a bin edge into the neighbouring bin; the candidates' exact distances
// (nn_d2) decide their order.
template <int DP>
__device__ __forceinline__ float nn_d2_dot(const float* q, float qn, const float* e, float en) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 4) {
        const float4 v = *reinterpret_cast<const float4*>(e + i);
        a0 = fmaf(q[i], v.x, a0);
        a1 = fmaf(q[i + 1], v.y, a1);
        a2 = fmaf(q[i + 2], v.z, a2);
        a3 = fmaf(q[i + 3], v.w, a3);
    }
    return fmaxf(fmaf(-2.f, (a0 + a1) + (a2 + a3), qn + en), 0.f);
}

// |q|^2 of a query held in registers (the same order in every kernel).
template <int DP>
__device__ __forceinline__ float nn_norm2(const float* q) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 4) {
        a0 = fmaf(q[i], q[i], a0);
        a1 = fmaf(q[i + 1], q[i + 1], a1);
        a2 = fmaf(q[i + 2], q[i + 2], a2);
        a3 = fmaf(q[i + 3], q[i + 3], a3);
    }
    return (a0 + a1) + (a2 + a3);
}

// Lower bound of the squared distance from a query to any entry of a tile:
// the distance to the tile's bounding box.
template <int DP>
__device__ __forceinline__ float nn_box_d2(const float* q, const float* lo, const float* hi) {
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 2) {
        const float g0 = fmaxf(fmaxf(lo[i] - q[i], q[i] - hi[i]), 0.f);
        const float g1 = fmaxf(fmaxf(lo[i + 1] - q[i + 1], q[i + 1] - hi[i + 1]), 0.f);
        a0 = fmaf(g0, g0, a0);
        a1 = fmaf(g1, g1, a1);
    }
    return a0 + a1;
}

// The same with the box read from global memory (every lane of a warp reads
// the same box, so the loads are broadcasts from L1).
template <int DP>
__device__ __forceinline__ float nn_box_d2_global(const float* q, const float* __restrict__ lo,
                                                  const float* __restrict__ hi) {
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 4) {
        const float4 l = __ldg(reinterpret_cast<const float4*>(lo + i));
        const float4 h = __ldg(reinterpret_cast<const float4*>(hi + i));
        const float g0 = fmaxf(fmaxf(l.x - q[i], q[i] - h.x), 0.f);
        const float g1 = fmaxf(fmaxf(l.y - q[i + 1], q[i + 1] - h.y), 0.f);
        const float g2 = fmaxf(fmaxf(l.z - q[i + 2], q[i + 2] - h.z), 0.f);
        const float g3 = fmaxf(fmaxf(l.w - q[i + 3], q[i + 3] - h.w), 0.f);
        a0 = fmaf(g0, g0, a0);
        a1 = fmaf(g1, g1, a1);
        a0 = fmaf(g2, g2, a0);
        a1 = fmaf(g3, g3, a1);
    }
    return a0 + a1;
}

#define NN_SUPER 32  // tiles whose boxes a CTA checks between two votes

// A tile whose box bound clears a distance limit by this margin holds no
// entry that nn_d2_dot puts below the limit (its rounding error is some
// 1e-7 of |q|^2 + |e|^2).
__device__ __forceinline__ bool nn_clears(float lb, float limit) {
    return lb > limit + 1e-3f + 1e-4f * limit;
}

// Float value where a query's fine bin b starts.
__device__ __forceinline__ float nn_bin_start(int base, int b) { return __uint_as_float((unsigned)(base + b - 1) << 19); }

// Load a tile of entries (coords, squared norms and hits) into shared memory.
template <int DP>
__device__ __forceinline__ void nn_load_tile(const NNArgs& a, int e0, int e_end, float* tile, int* thits,
                                             float* ten) {
    const int n = min(NN_TE, e_end - e0);
    const float4* src = reinterpret_cast<const float4*>(a.coords + (long)e0 * DP);
    float4* dst = reinterpret_cast<float4*>(tile);
    for (int i = threadIdx.x; i < NN_TE * DP / 4; i += blockDim.x)
        dst[i] = (i < n * DP / 4) ? src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = threadIdx.x; i < NN_TE; i += blockDim.x) {
        thits[i] = i < n ? a.hits[e0 + i] : 0;
        ten[i] = i < n ? a.enorm[e0 + i] : 0.f;
    }
}

// A thread's queries are NN_QPT consecutive (sorted) slots, so a warp holds
// 32 NN_QPT similar reads; its histogram rows sit at row j * NN_THREADS + tid
// (bank-conflict free).  Per tile of 32 entries, each query first bounds
// its distance to the tile's box: a tile beyond the start of the query's
// last bin (open-ended, far beyond its k-hit radius) adds its hits to that
// bin at once; the CTA loads the tile only if some query needs it, and a
// warp whose queries all clear it skips the distances.
template <int DP>
__global__ void __launch_bounds__(NN_THREADS) wp_nn_hist_kernel(NNArgs a) {
    extern __shared__ __align__(16) unsigned char nn_smem[];
    float* tile = reinterpret_cast<float*>(nn_smem);
    int* thits = reinterpret_cast<int*>(tile + NN_TE * DP);
    float* ten = reinterpret_cast<float*>(thits + NN_TE);
    float* box = ten + NN_TE;                                    // [2][DP]
    unsigned* hist = reinterpret_cast<unsigned*>(box + 2 * DP);  // [NN_QPB][NN_NB + 1]
    const int qb = blockIdx.x * NN_QPB;
    // entry slice s, or with sub-slices part p of it (whole super-tiles)
    const int sub = a.sub > 1 ? a.sub : 1;
    const int s = blockIdx.y / sub, part = blockIdx.y % sub;
    const int slice0 = s * a.slice_len;
    const int nsps = (a.slice_len + NN_TE * NN_SUPER - 1) / (NN_TE * NN_SUPER);  // super-tiles per slice
    int e_lo = slice0, e_hi = min(a.N, e_lo + a.slice_len);
    if (sub > 1) {
        const int st = (e_hi - e_lo + NN_TE * NN_SUPER - 1) / (NN_TE * NN_SUPER);  // super-tiles in the slice
        const int a0 = (int)((long)st * part / sub), a1 = (int)((long)st * (part + 1) / sub);
        const int lo = e_lo;
        e_lo = min(e_hi, lo + a0 * NN_TE * NN_SUPER);
        e_hi = min(e_hi, lo + a1 * NN_TE * NN_SUPER);
    }
    for (int i = threadIdx.x; i < NN_QPB * (NN_NB + 1); i += blockDim.x) hist[i] = 0u;
    float q[NN_QPT][DP];
    bool valid[NN_QPT];
    int base[NN_QPT];
    float far[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) {
        const int lq = threadIdx.x * NN_QPT + j;
        valid[j] = qb + lq < a.R;
        const int slot = !valid[j] ? 0 : (a.slots ? a.slots[qb + lq] : qb + lq);
        const float* src = a.queries + (long)slot * DP;
#pragma unroll
        for (int i = 0; i < DP; i++) q[j][i] = valid[j] ? src[i] : 0.f;
        base[j] = valid[j] ? a.qbase[a.q0 + slot] : 0;
        far[j] = valid[j] ? nn_bin_start(base[j], NN_NB - 1) : INFINITY;
    }
    float qn[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) qn[j] = nn_norm2<DP>(q[j]);
    unsigned* vote = reinterpret_cast<unsigned*>(box);
    for (int st0 = e_lo; st0 < e_hi; st0 += NN_TE * NN_SUPER) {
        // which of the next NN_SUPER tiles each read needs; the others add
        // their hits to the read's open last bin
        const int t0 = st0 / NN_TE, nt = min(NN_SUPER, (e_hi - st0 + NN_TE - 1) / NN_TE);
        unsigned nm[NN_QPT];
        int mb[NN_QPT];  // smallest bin of the read's entries in this super-tile
#pragma unroll
        for (int j = 0; j < NN_QPT; j++) {
            nm[j] = 0u;
            mb[j] = NN_NB - 1;
        }
        for (int tt = 0; tt < nt; tt++) {
            const long t = t0 + tt;
#pragma unroll
            for (int j = 0; j < NN_QPT; j++) {
                if (!valid[j]) continue;
                if (!nn_clears(nn_box_d2_global<DP>(q[j], a.tlo + t * DP, a.thi + t * DP), far[j]))
                    nm[j] |= 1u << tt;
                else
                    atomicAdd(&hist[(j * NN_THREADS + threadIdx.x) * (NN_NB + 1) + NN_NB - 1], (unsigned)a.ttot[t]);
            }
        }
        unsigned wm = 0u;
#pragma unroll
        for (int j = 0; j < NN_QPT; j++) wm |= nm[j];
        wm = __reduce_or_sync(0xffffffffu, wm);
        __syncthreads();
        if (threadIdx.x == 0) vote[0] = 0u;
        __syncthreads();
        if ((threadIdx.x & 31) == 0 && wm) atomicOr(&vote[0], wm);
        __syncthreads();
        unsigned cm = vote[0];
        while (cm) {
            const int tt = __ffs(cm) - 1;
            cm &= cm - 1;
            const int e0 = st0 + tt * NN_TE;
            __syncthreads();
            nn_load_tile<DP>(a, e0, e_hi, tile, thits, ten);
            __syncthreads();
            if (!((wm >> tt) & 1u)) continue;
            bool need[NN_QPT];
#pragma unroll
            for (int j = 0; j < NN_QPT; j++) need[j] = (nm[j] >> tt) & 1u;
            const int n = min(NN_TE, e_hi - e0);
            for (int e = 0; e < n; e++) {
#pragma unroll
                for (int j = 0; j < NN_QPT; j++) {
                    const float d2 = nn_d2_dot<DP>(q[j], qn[j], tile + e * DP, ten[e]);
                    if (need[j]) {
                        const int bin = nn_bin(d2, base[j]);
                        mb[j] = min(mb[j], bin);
                        atomicAdd(&hist[(j * NN_THREADS + threadIdx.x) * (NN_NB + 1) + bin], (unsigned)thits[e]);
                    }
                }
            }
        }
        if (a.stmin) {
            const int sti = s * nsps + (st0 - slice0) / (NN_TE * NN_SUPER);
#pragma unroll
            for (int j = 0; j < NN_QPT; j++) {
                const int lq = threadIdx.x * NN_QPT + j;
                if (!valid[j]) continue;
                const int slot = a.slots ? a.slots[qb + lq] : qb + lq;
                a.stmin[(long)(a.q0 + slot) * a.n_super + sti] = (unsigned char)mb[j];
            }
        }
    }
    __syncthreads();
    // this slice's histograms, query-major within the slice
    for (int i = threadIdx.x; i < NN_QPB * NN_NB; i += blockDim.x) {
        const int lq = i / NN_NB, b = i % NN_NB;
        const int row = (lq % NN_QPT) * NN_THREADS + lq / NN_QPT;
        if (qb + lq < a.R) {
            const int slot = a.slots ? a.slots[qb + lq] : qb + lq;
            unsigned* dst = &a.shist[((long)s * a.R_all + a.q0 + slot) * NN_NB + b];
            const unsigned v = hist[row * (NN_NB + 1) + b];
            if (sub > 1) {
                if (v) atomicAdd(dst, v);
            } else {
                *dst = v;
            }
        }
    }
}

// Per query: where its k-hit radius lies, from a sample of the entries
// drawn in proportion to their hits (systematic sampling of the cumulative
// hits, so each sample point stands for the same number of hits): the
// k-hit radius is the k / (all hits) quantile of the hits-weighted
// distances, estimated by the sample's ceil(k x sample_n / all hits)-th
// nearest point (binned coarsely); the query's fine bins start 3 3/8
// octaves below that coarse bin and end, with the open last bin, half an
// octave above it.  Only the bins move with the estimate; the
// selection stays exact whatever it says (a poor estimate only leaves more
// candidates).
template <int DP>
__global__ void __launch_bounds__(NN_THREADS) wp_nn_estimate_kernel(NNArgs a) {
    extern __shared__ __align__(16) unsigned char nn_smem[];
    float* tile = reinterpret_cast<float*>(nn_smem);
    int* thits = reinterpret_cast<int*>(tile + NN_TE * DP);
    float* ten = reinterpret_cast<float*>(thits + NN_TE);
    unsigned* hist = reinterpret_cast<unsigned*>(ten + NN_TE);  // [NN_QPB][NN_NB + 1]
    const int qb = blockIdx.x * NN_QPB;
    for (int i = threadIdx.x; i < NN_QPB * (NN_NB + 1); i += blockDim.x) hist[i] = 0u;
    float q[NN_QPT][DP];
    bool valid[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) {
        const int lq = threadIdx.x * NN_QPT + j;
        valid[j] = qb + lq < a.R;
        const float* src = a.queries + (long)(valid[j] ? qb + lq : 0) * DP;
#pragma unroll
        for (int i = 0; i < DP; i++) q[j][i] = valid[j] ? src[i] : 0.f;
    }
    float qn[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) qn[j] = nn_norm2<DP>(q[j]);
    for (int s0 = 0; s0 < a.sample_n; s0 += NN_TE) {
        __syncthreads();
        const int n = min(NN_TE, a.sample_n - s0);
        for (int i = threadIdx.x; i < NN_TE * DP / 4; i += blockDim.x) {
            const int e = i / (DP / 4), part = i % (DP / 4);
            reinterpret_cast<float4*>(tile)[i] =
                e < n ? reinterpret_cast<const float4*>(a.coords + (long)a.sample[s0 + e] * DP)[part]
                      : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int i = threadIdx.x; i < NN_TE; i += blockDim.x) ten[i] = i < n ? a.enorm[a.sample[s0 + i]] : 0.f;
        __syncthreads();
        for (int e = 0; e < n; e++) {
#pragma unroll
            for (int j = 0; j < NN_QPT; j++) {
                const float d2 = nn_d2_dot<DP>(q[j], qn[j], tile + e * DP, ten[e]);
                if (valid[j]) atomicAdd(&hist[(threadIdx.x + j * NN_THREADS) * (NN_NB + 1) + nn_coarse_bin(d2)], 1u);
            }
        }
    }
    __syncthreads();
    // the sample point that stands for the k-th hit
    const long long kth = (a.k * a.sample_n + a.hits_total - 1) / a.hits_total;
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) {
        if (!valid[j]) continue;
        const unsigned* h = hist + (threadIdx.x + j * NN_THREADS) * (NN_NB + 1);
        long long run = 0;
        int b = NN_NB - 1;
        for (int i = 0; i < NN_NB; i++) {
            run += h[i];
            if (run >= kth) {
                b = i;
                break;
            }
        }
        // coarse bin b starts at float bits >> 21 == b - 1 + ((127 - 6) << 2);
        // the fine bins start 54 sixteenths of an octave below it, so the
        // last (open) fine bin starts half an octave above it (a read whose
        // radius lies beyond is counted again with its bins moved up,
        // wp_nn_redo_kernel)
        const int ck = b - 1 + ((127 - 6) << 2);
        a.qbase[a.q0 + qb + threadIdx.x * NN_QPT + j] = 4 * ck - 54;
    }
}

// Per query: the slices' histograms summed, the bin b* where the running
// hits reach k, hits below it, the candidate bound, and each slice's share
// (offsets of the slices inside the query's list).
__global__ void wp_nn_threshold_kernel(NNArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.R) return;
    const int gq = a.q0 + (a.slots ? a.slots[q] : q);
    long long cum = 0, below = 0, cap = 0;
    int b = NN_NB - 1;
    bool found = false;
    // The reference's k-hit set: b* is the bin holding the final top's
    // distance plus the binning distance's rounding (the margin of
    // nn_clears), or the open last bin when every entry is kept.
    int bound_bin = -1;
    if (a.tf_d) {
        const double td = a.tf_d[gq];
        bound_bin = (a.tf_flag[gq] & 1) ? NN_NB - 1
                                         : nn_bin((float)(td * (1.0 + 1e-4) + 1e-3) * (1.f + 1e-6f), a.qbase[gq]);
    }
    for (int i = 0; i < NN_NB; i++) {
        long long hi = 0;
        for (int s = 0; s < a.slices; s++) hi += a.shist[((long)s * a.R_all + gq) * NN_NB + i];
        if (!found && (bound_bin >= 0 ? i == bound_bin : cum + hi >= a.k)) {
            found = true;
            b = i;
            below = cum;
            cap = cum + hi;
        }
        cum += hi;
    }
    if (!found) {  // all hits stay below k: every entry is kept
        long long hl = 0;
        for (int s = 0; s < a.slices; s++) hl += a.shist[((long)s * a.R_all + gq) * NN_NB + NN_NB - 1];
        b = NN_NB - 1;
        below = cum - hl;
        cap = cum;
    }
    a.qbin[gq] = b;
    a.qbelow[gq] = (int)below;
    a.qcap[gq] = cap;
    long long off = 0;
    for (int s = 0; s < a.slices; s++) {
        long long c = 0;
        for (int i = 0; i <= b; i++) c += a.shist[((long)s * a.R_all + gq) * NN_NB + i];
        a.sliceoff[(long)s * a.R_all + gq] = off;
        a.slicecap[(long)s * a.R_all + gq] = c;
        off += c;
    }
}

template <int DP>
__global__ void __launch_bounds__(NN_THREADS) wp_nn_collect_kernel(NNArgs a) {
    extern __shared__ __align__(16) unsigned char nn_smem[];
    float* tile = reinterpret_cast<float*>(nn_smem);
    int* thits = reinterpret_cast<int*>(tile + NN_TE * DP);
    float* ten = reinterpret_cast<float*>(thits + NN_TE);
    float* box = ten + NN_TE;  // [2][DP]
    const int qb = blockIdx.x * NN_QPB;
    const int s = blockIdx.y;
    const int e_lo = s * a.slice_len, e_hi = min(a.N, e_lo + a.slice_len);
    const int nsps = (a.slice_len + NN_TE * NN_SUPER - 1) / (NN_TE * NN_SUPER);
    float q[NN_QPT][DP];
    bool valid[NN_QPT];
    int bstar[NN_QPT], base[NN_QPT];
    float lim[NN_QPT];
    long long off[NN_QPT], cap[NN_QPT], cnt[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) {
        const int lq = threadIdx.x * NN_QPT + j;
        valid[j] = qb + lq < a.R;
        const int l = valid[j] ? qb + lq : 0;
        const int gq = a.q0 + l;
        const float* src = a.queries + (long)l * DP;
#pragma unroll
        for (int i = 0; i < DP; i++) q[j][i] = valid[j] ? src[i] : 0.f;
        bstar[j] = valid[j] ? a.qbin[gq] : -1;
        base[j] = valid[j] ? a.qbase[gq] : 0;
        off[j] = valid[j] ? a.qoff[l] + a.sliceoff[(long)s * a.R_all + gq] : 0;
        cap[j] = valid[j] ? a.slicecap[(long)s * a.R_all + gq] : 0;
        cnt[j] = 0;
        // candidates lie below the start of bin b* + 1 (none beyond the open last bin)
        lim[j] = !valid[j] ? -1.f : (bstar[j] >= NN_NB - 1 ? INFINITY : nn_bin_start(base[j], bstar[j] + 1));
    }
    float qn[NN_QPT];
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) qn[j] = nn_norm2<DP>(q[j]);
    unsigned* vote = reinterpret_cast<unsigned*>(box);
    for (int st0 = e_lo; st0 < e_hi; st0 += NN_TE * NN_SUPER) {
        const int t0 = st0 / NN_TE, nt = min(NN_SUPER, (e_hi - st0 + NN_TE - 1) / NN_TE);
        // reads with no entry at or below b* in this super-tile (the
        // histogram pass's smallest bin) need none of its tiles
        bool sn[NN_QPT];
        const int sti = s * nsps + (st0 - e_lo) / (NN_TE * NN_SUPER);
#pragma unroll
        for (int j = 0; j < NN_QPT; j++) {
            const int lq = threadIdx.x * NN_QPT + j;
            sn[j] = valid[j] && (!a.stmin || (int)a.stmin[(long)(a.q0 + qb + lq) * a.n_super + sti] <= bstar[j]);
        }
        unsigned wm = 0u;
        for (int tt = 0; tt < nt; tt++) {
            const long t = t0 + tt;
            bool nd = false;
#pragma unroll
            for (int j = 0; j < NN_QPT; j++)
                nd |= sn[j] && !nn_clears(nn_box_d2_global<DP>(q[j], a.tlo + t * DP, a.thi + t * DP), lim[j]);
            if (nd) wm |= 1u << tt;
        }
        wm = __reduce_or_sync(0xffffffffu, wm);
        __syncthreads();
        if (threadIdx.x == 0) vote[0] = 0u;
        __syncthreads();
        if ((threadIdx.x & 31) == 0 && wm) atomicOr(&vote[0], wm);
        __syncthreads();
        unsigned cm = vote[0];
        while (cm) {
        const int tt = __ffs(cm) - 1;
        cm &= cm - 1;
        const int e0 = st0 + tt * NN_TE;
        __syncthreads();
        nn_load_tile<DP>(a, e0, e_hi, tile, thits, ten);
        __syncthreads();
        if (!((wm >> tt) & 1u)) continue;
        const int n = min(NN_TE, e_hi - e0);
        for (int e = 0; e < n; e++) {
#pragma unroll
            for (int j = 0; j < NN_QPT; j++) {
                const int bin = nn_bin(nn_d2_dot<DP>(q[j], qn[j], tile + e * DP, ten[e]), base[j]);
                if (bin <= bstar[j]) {
                    if (cnt[j] < cap[j]) {
                        a.cand_idx[off[j] + cnt[j]] = e0 + e;
                        a.cand_d2[off[j] + cnt[j]] = nn_d2<DP>(q[j], tile + e * DP);
                        a.cand_hits[off[j] + cnt[j]] = thits[e];
                        a.cand_bin[off[j] + cnt[j]] = (unsigned char)bin;
                    } else {
                        atomicExch(a.err, 1);
                    }
                    cnt[j]++;
                }
            }
        }
        }
    }
#pragma unroll
    for (int j = 0; j < NN_QPT; j++) {
        if (!valid[j]) continue;
        a.slicecnt[(long)s * a.R_all + a.q0 + qb + threadIdx.x * NN_QPT + j] = cnt[j];
        if (cnt[j] > cap[j]) atomicExch(a.err, 1);
    }
}


__device__ __forceinline__ unsigned long long nn_dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Warp-wide inclusive prefix sum.
__device__ __forceinline__ long long warp_incl_scan(long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Radix-select step over a warp's 256-digit histogram, counting from digit
// 255 down: the digit where the running count reaches `want`; *before gets
// the count of the digits above it.  Lane l scans digits [248 - 8l, 256 - 8l).
__device__ int nn_digit_from_top(const unsigned long long* hist, long long want, long long* before_out) {
    const int lane = threadIdx.x & 31;
    long long mine = 0;
    for (int i = 0; i < 8; i++) mine += (long long)hist[255 - (lane * 8 + i)];
    const long long incl = warp_incl_scan(mine);
    const unsigned hit = __ballot_sync(0xffffffffu, incl >= want);
    const int L = __ffs(hit) - 1;
    long long before = __shfl_sync(0xffffffffu, incl - mine, L);
    int digit = 0;
    if (lane == L) {
        long long c = before;
        for (int i = 0; i < 8; i++) {
            const int d = 255 - (L * 8 + i);
            const long long hb = (long long)hist[d];
            if (c + hb >= want) {
                digit = d;
                break;
            }
            c += hb;
        }
        before = c;
    }
    *before_out = __shfl_sync(0xffffffffu, before, L);
    return __shfl_sync(0xffffffffu, digit, L);
}

__global__ void __launch_bounds__(NN_SEL_WARPS * 32) wp_nn_select_kernel(NNSelectArgs a) {
    extern __shared__ __align__(16) unsigned char nn_sel_smem[];
    unsigned long long(*s_hist)[256] = reinterpret_cast<unsigned long long(*)[256]>(nn_sel_smem);
    double(*s_key)[NN_HMAX] = reinterpret_cast<double(*)[NN_HMAX]>(nn_sel_smem + sizeof(unsigned long long) * 256 * NN_SEL_WARPS);
    int(*s_id)[NN_HMAX] = reinterpret_cast<int(*)[NN_HMAX]>(nn_sel_smem + sizeof(unsigned long long) * 256 * NN_SEL_WARPS
                                                              + sizeof(double) * NN_HMAX * NN_SEL_WARPS);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const long gw = (long)blockIdx.x * NN_SEL_WARPS + wib;
    const long nw = (long)gridDim.x * NN_SEL_WARPS;
    double* acc = a.acc + gw * a.U;
    int* mark = a.mark + gw * a.U;
    int* touched = a.touched + gw * a.U;
    unsigned long long* hist = s_hist[wib];

    for (long lq = gw; lq < a.R; lq += nw) {
        const int gq = a.q0 + (int)lq;
        const int bstar = a.qbin[gq];
        long long need = a.k - a.qbelow[gq];  // hits still needed from bin b*
        // the reference's k-hit set: entries at or below the replayed final
        // top (FP64 distance, tree position); FP32 distances decide unless
        // they lie within their rounding margin of the top's
        const bool exact = a.tf_d != nullptr;
        const double tf_d = exact ? a.tf_d[gq] : 0.0;
        const int tf_pos = exact ? a.tf_pos[gq] : 0;
        const bool tf_all = exact && (a.tf_flag[gq] & 1);
        const double tf_m = 2e-5 * tf_d + 1e-3;
        const double* q64 = exact ? a.rads + (long)(a.qperm ? a.qperm[gq] : gq) * a.TC : nullptr;
        unsigned kstar_out = 0u;
        bool take_all_out = false;
        if (!exact) {
        // The query's candidates: one segment per entry slice, in slice
        // order (so in ascending entry index overall).

        // ---- hits-weighted radix select over the float bits of d2 in bin b*.
        // the keys of bin b*'s candidates share their top bits: the radix
        // passes start below the common prefix of the smallest and largest
        unsigned kmin = 0xffffffffu, kmax = 0u;
        for (int sl = 0; sl < a.slices; sl++) {
            const long long sb = a.qoff[lq] + a.sliceoff[(long)sl * a.R_all + gq];
            const long long sn = min(a.slicecnt[(long)sl * a.R_all + gq], a.slicecap[(long)sl * a.R_all + gq]);
            for (long long i = lane; i < sn; i += 32)
                if (a.cand_bin[sb + i] == bstar) {
                    const unsigned key = __float_as_uint(a.cand_d2[sb + i]);
                    kmin = min(kmin, key);
                    kmax = max(kmax, key);
                }
        }
        for (int o = 16; o > 0; o >>= 1) {
            kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
            kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
        }
        const int common = kmin <= kmax ? __clz((int)(kmin ^ kmax)) : 32;  // 32 when all keys are equal
        const int rem = 32 - common;
        unsigned pmask = common >= 32 ? 0xffffffffu : (common == 0 ? 0u : ~0u << rem);
        unsigned prefix = kmin & pmask;
        bool take_all = false;
        for (int shift = rem > 8 ? rem - 8 : 0;; shift = shift > 8 ? shift - 8 : 0) {
            for (int i = lane; i < 256; i += 32) hist[i] = 0ull;
            __syncwarp();
            for (int sl = 0; sl < a.slices; sl++) {
                const long long sb = a.qoff[lq] + a.sliceoff[(long)sl * a.R_all + gq];
                const long long sn = min(a.slicecnt[(long)sl * a.R_all + gq], a.slicecap[(long)sl * a.R_all + gq]);
                for (long long i = lane; i < sn; i += 32) {
                    const unsigned key = __float_as_uint(a.cand_d2[sb + i]);
                    if (a.cand_bin[sb + i] == bstar && (key & pmask) == prefix)
                        atomicAdd(&hist[(key >> shift) & 255u], (unsigned long long)a.cand_hits[sb + i]);
                }
            }
            __syncwarp();
            // find the digit where the running hits reach `need`
            long long tot = 0;
            for (int i = lane; i < 256; i += 32) tot += (long long)hist[i];
            for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
            if (tot < need) {
                take_all = true;  // hits of this prefix never reach k: keep them all
                break;
            }
            // lane l covers digits [8l, 8l + 8)
            long long mine = 0;
            for (int i = 0; i < 8; i++) mine += (long long)hist[lane * 8 + i];
            const long long incl = warp_incl_scan(mine);
            const unsigned hit = __ballot_sync(0xffffffffu, incl >= need);
            const int L = __ffs(hit) - 1;
            long long before = __shfl_sync(0xffffffffu, incl - mine, L);
            int digit = 0;
            if (lane == L) {
                long long c = before;
                for (int i = 0; i < 8; i++) {
                    const long long hb = (long long)hist[L * 8 + i];
                    if (c + hb >= need) {
                        digit = L * 8 + i;
                        break;
                    }
                    c += hb;
                }
                before = c;
            }
            digit = __shfl_sync(0xffffffffu, digit, L);
            before = __shfl_sync(0xffffffffu, before, L);
            need -= before;
            prefix |= (unsigned)digit << shift;
            pmask |= 255u << shift;
            __syncwarp();
            if (shift == 0) break;
        }
        kstar_out = prefix;
        take_all_out = take_all;
        }
        const bool take_all = exact ? tf_all : take_all_out;
        const unsigned kstar = kstar_out;  // with take_all: unused
        // Weights of the entries near the read (within 18.5 x 2 sig^2 of the
        // nearest, i.e. above 1e-8 of the largest weight) from FP64
        // distances, as the reference forms them; the far ones from FP32
        // (their error is below 1e-8 of the largest weight).
        float dmin = INFINITY;
        if (a.rads) {
            for (int sl = 0; sl < a.slices; sl++) {
                const long long sb = a.qoff[lq] + a.sliceoff[(long)sl * a.R_all + gq];
                const long long sn = min(a.slicecnt[(long)sl * a.R_all + gq], a.slicecap[(long)sl * a.R_all + gq]);
                for (long long i = lane; i < sn; i += 32) dmin = fminf(dmin, a.cand_d2[sb + i]);
            }
            for (int o = 16; o > 0; o >>= 1) dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
        }
        const double wlim = (double)dmin + 18.5 * a.two_sig_sq + 1e-3;
        const double* qw = a.rads ? a.rads + (long)(a.qperm ? a.qperm[gq] : gq) * a.TC : nullptr;
        // ---- contributions of the kept entries, in candidate (entry) order.
        double total_part = 0.0;
        int ntouched = 0;
        long long tie_cum = 0;  // hits of key == kstar entries seen so far
        for (int sl = 0; sl < a.slices; sl++) {
          const long long sb = a.qoff[lq] + a.sliceoff[(long)sl * a.R_all + gq];
          const long long sn = min(a.slicecnt[(long)sl * a.R_all + gq], a.slicecap[(long)sl * a.R_all + gq]);
          for (long long i0 = 0; i0 < sn; i0 += 32) {
            const long long i = i0 + lane;
            bool keep = false;
            int e = -1;
            float d2 = 0.f;
            bool tie = false;
            if (i < sn) {
                e = a.cand_idx[sb + i];
                d2 = a.cand_d2[sb + i];
                const int b = a.cand_bin[sb + i];
                const unsigned key = __float_as_uint(d2);
                if (take_all) keep = true;
                else if (exact) {
                    if ((double)d2 < tf_d - tf_m) keep = true;
                    else if ((double)d2 <= tf_d + tf_m) {
                        const double d64 = wp_nn_exact_d2(q64, e, a.TC, a.C, a.DP, a.cnt, a.ctab, a.NC, a.ecoord);
                        keep = d64 < tf_d || (d64 == tf_d && e <= tf_pos);
                    }
                } else if (b < bstar) keep = true;
                else if (key < kstar) keep = true;
                else if (key == kstar) tie = true;
            }
            // ties at kstar: keep in entry order while the tie hits before
            // this one are below `need`
            const long long th = tie ? (long long)a.cand_hits[sb + i] : 0;
            const long long incl = warp_incl_scan(th);
            if (tie && tie_cum + incl - th < need) keep = true;
            tie_cum += __shfl_sync(0xffffffffu, incl, 31);
            // exp(-d2 / 2 sig^2) as 2^x: exp2f of the fraction, the integer
            // part applied in FP64 so far entries keep a non-zero weight
            double w = 0.0;
            if (keep) {
                if (qw && (double)d2 < wlim) {
                    const double d64 = wp_nn_exact_d2(qw, e, a.TC, a.C, a.DP, a.cnt, a.ctab, a.NC, a.ecoord);
                    w = exp(-d64 / a.two_sig_sq);
                } else {
                    const float x = -d2 * a.inv_two_sig_sq * 1.4426950408889634f;
                    const float fl = floorf(x);
                    w = ldexp((double)exp2f(x - fl), (int)fl);
                }
            }
            const int s0 = keep ? a.src_off[e] : 0;
            const int ns = keep ? a.src_off[e + 1] - s0 : 0;
            // the kept entries' sources, flattened over the warp: source j of
            // this batch belongs to the first lane whose inclusive prefix of
            // source counts exceeds j (a popular track's many sources no
            // longer hold the other lanes idle)
            int pre = ns;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, pre, o);
                if (lane >= o) pre += t;
            }
            const int nsrc = __shfl_sync(0xffffffffu, pre, 31);
            const int excl = pre - ns;
            for (int j0 = 0; j0 < nsrc; j0 += 32) {
                const int j = j0 + lane;
                const bool act = j < nsrc;
                int L = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(0xffffffffu, pre, L + step - 1) <= j) L += step;
                const int sL = __shfl_sync(0xffffffffu, s0, L) + j - __shfl_sync(0xffffffffu, excl, L);
                const double wL = __shfl_sync(0xffffffffu, w, L);
                int id = -1;
                double val = 0.0;
                if (act) {
                    id = a.src_dense[sL];
                    val = wL * a.src_ratio[sL];
                    total_part += wL * (double)a.src_hits[sL];
                }
                const unsigned actm = __ballot_sync(0xffffffffu, act);
                if (actm == 0u) continue;
                const unsigned grp = __match_any_sync(0xffffffffu, id);
                // group sum in lane order, at the group's lowest lane
                double gsum = 0.0;
                unsigned gm = grp;
                while (gm) {
                    const int src = __ffs(gm) - 1;
                    gm &= gm - 1;
                    const double v = __shfl_sync(grp, val, src);
                    gsum += v;
                }
                const bool leader = act && lane == __ffs(grp) - 1;
                const bool fresh = leader && mark[id] == 0;
                const unsigned fm = __ballot_sync(0xffffffffu, fresh);
                if (fresh) {
                    mark[id] = 1;
                    touched[ntouched + __popc(fm & ((1u << lane) - 1u))] = id;
                }
                if (leader) acc[id] += gsum;
                ntouched += __popc(fm);
                __syncwarp();
            }
          }
        }
        // total, summed in a fixed tree order and broadcast from lane 0
        double tot = total_part;
        for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
        tot = __shfl_sync(0xffffffffu, tot, 0);

        // ---- top h of the touched ids by (score, id).
        const int h = a.h;
        int nsel = 0;
        unsigned long long sthr = 0ull;  // keep ids with score bits > sthr, ties by id
        int tie_keep = 0;                 // how many score == sthr ids to keep (largest ids)
        bool all = ntouched <= h;
        if (!all) {
            // radix select of the h-th largest score (count based, 8 passes)
            unsigned long long pre = 0ull, msk = 0ull;
            long long want = h;  // from the top
            for (int pass = 0; pass < 8; pass++) {
                const int shift = 56 - 8 * pass;
                for (int i = lane; i < 256; i += 32) hist[i] = 0ull;
                __syncwarp();
                for (int i = lane; i < ntouched; i += 32) {
                    const unsigned long long kb = nn_dbits(acc[touched[i]]);
                    if ((kb & msk) == pre) atomicAdd(&hist[(kb >> shift) & 255ull], 1ull);
                }
                __syncwarp();
                long long before = 0;
                const int digit = nn_digit_from_top(hist, want, &before);
                want -= before;
                pre |= (unsigned long long)digit << shift;
                msk |= 255ull << shift;
                __syncwarp();
            }
            sthr = pre;
            tie_keep = (int)want;  // ids with score == sthr to keep, largest ids first
        }
        // the tie_keep largest ids among those scoring exactly sthr: a radix
        // select on the (distinct, non-negative) dense ids
        int id_thr = 0x7fffffff;
        if (!all && tie_keep > 0) {
            unsigned pre2 = 0u, msk2 = 0u;
            long long want2 = tie_keep;
            for (int pass = 0; pass < 4; pass++) {
                const int shift = 24 - 8 * pass;
                for (int i = lane; i < 256; i += 32) hist[i] = 0ull;
                __syncwarp();
                for (int i = lane; i < ntouched; i += 32) {
                    const unsigned id = (unsigned)touched[i];
                    if (nn_dbits(acc[id]) == sthr && (id & msk2) == pre2) atomicAdd(&hist[(id >> shift) & 255u], 1ull);
                }
                __syncwarp();
                long long before = 0;
                const int digit = nn_digit_from_top(hist, want2, &before);
                want2 -= before;
                pre2 |= (unsigned)digit << shift;
                msk2 |= 255u << shift;
                __syncwarp();
            }
            id_thr = (int)pre2;
        }
        // gather the kept ids into shared memory (order fixed below by sort)
        for (int base = 0; base < ntouched; base += 32) {
            const int i = base + lane;
            bool sel = false;
            int id = 0;
            double sc = 0.0;
            if (i < ntouched) {
                id = touched[i];
                sc = acc[id];
                if (all) sel = true;
                else {
                    const unsigned long long kb = nn_dbits(sc);
                    if (kb > sthr) sel = true;
                    else if (kb == sthr) sel = id >= id_thr;
                }
            }
            const unsigned sm = __ballot_sync(0xffffffffu, sel);
            if (sel) {
                const int pos = nsel + __popc(sm & ((1u << lane) - 1u));
                s_key[wib][pos] = sc;
                s_id[wib][pos] = id;
            }
            nsel += __popc(sm);
        }
        __syncwarp();
        // bitonic sort ascending by (score, id) over the next power of two
        int n2 = 1;
        while (n2 < nsel) n2 <<= 1;
        for (int i = nsel + lane; i < n2; i += 32) {
            s_key[wib][i] = INFINITY;
            s_id[wib][i] = 0x7fffffff;
        }
        __syncwarp();
        for (int size = 2; size <= n2; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = lane; i < n2; i += 32) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const bool up = (i & size) == 0;
                        const double ki = s_key[wib][i], kj = s_key[wib][j];
                        const int ii = s_id[wib][i], ij = s_id[wib][j];
                        const bool gt = ki > kj || (ki == kj && ii > ij);
                        if (gt == up) {
                            s_key[wib][i] = kj;
                            s_key[wib][j] = ki;
                            s_id[wib][i] = ij;
                            s_id[wib][j] = ii;
                        }
                    }
                }
                __syncwarp();
            }
        }
        // outputs, at the read's own index
        const int oq = a.qperm ? a.qperm[gq] : gq;
        for (int i = lane; i < nsel; i += 32) {
            const int u = s_id[wib][i];
            a.out_cand_id[(long)oq * h + i] = a.dense_id[u];
            a.out_cand_score[(long)oq * h + i] = s_key[wib][i];
            if (a.out_cand_pep) a.out_cand_pep[(long)oq * h + i] = a.dense_pep[u];
        }
        if (a.out_subfrac) {
            // HybridClassifier: sum of adjusted score x peptide count, in
            // candidate order (hybrid-classifier.cc:58-64); the terms formed
            // in parallel, summed in order by one lane
            __syncwarp();
            for (int i = lane; i < nsel; i += 32)
                s_key[wib][i] = (s_key[wib][i] / tot) * (double)a.dense_count[s_id[wib][i]];
            __syncwarp();
            if (lane == 0) {
                double sf = 0.0;
                for (int i = 0; i < nsel; i++) sf += s_key[wib][i];
                a.out_subfrac[oq] = sf;
            }
        }
        if (lane == 0) {
            a.out_ncand[oq] = nsel;
            a.out_total[oq] = tot;
        }
        __syncwarp();
        // reset the per-warp accumulators
        for (int i = lane; i < ntouched; i += 32) {
            const int id = touched[i];
            acc[id] = 0.0;
            mark[id] = 0;
        }
        __syncwarp();
    }
}

// Queries as FP32 rows padded to DP (zeros beyond T * C).
__global__ void wp_nn_queries_kernel(const double* __restrict__ rads, int R, int TC, int DP,
                                     float* __restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)R * DP) return;
    const long r = i / DP;
    const int d = (int)(i % DP);
    out[i] = d < TC ? (float)rads[r * TC + d] : 0.f;
}

// Gather [R][h] candidate lists into one ragged array (offsets given).
__global__ void wp_nn_ragged_kernel(const int* __restrict__ cand, int h, const int* __restrict__ off, int R,
                                    int* __restrict__ out) {
    const int r = blockIdx.x;
    if (r >= R) return;
    const int n = off[r + 1] - off[r];
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[off[r] + i] = cand[(long)r * h + i];
}

// HybridClassifier::classify's last steps (hybrid-classifier.cc:66-79): the
// HMM score times the subfraction, NaN patched; no candidate: (-1, 0, 1).
__global__ void wp_hybrid_finish_kernel(const int* __restrict__ ncand, const double* __restrict__ subfrac, int R,
                                        int* __restrict__ id, double* __restrict__ score,
                                        double* __restrict__ total) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    if (ncand[r] == 0) {
        id[r] = -1;
        score[r] = 0.0;
        total[r] = 1.0;
        return;
    }
    const double s = score[r] * subfrac[r];
    if (isnan(s / total[r])) {
        score[r] = 0.0;
        total[r] = 1.0;
    } else {
        score[r] = s;
    }
}

cudaError_t wp_launch_hybrid_finish(const int* ncand, const double* subfrac, int R, int* id, double* score,
                                    double* total, cudaStream_t s) {
    if (R == 0) return cudaSuccess;
    wp_hybrid_finish_kernel<<<(R + 255) / 256, 256, 0, s>>>(ncand, subfrac, R, id, score, total);
    return cudaGetLastError();
}

size_t wp_nn_dist_smem_bytes(int DP, bool with_hist) {
    size_t b = sizeof(float) * NN_TE * DP + sizeof(int) * NN_TE + sizeof(float) * NN_TE + sizeof(float) * 2 * DP;
    if (with_hist) b += sizeof(unsigned) * NN_QPB * (NN_NB + 1);
    return b;
}

int wp_nn_bins() { return NN_NB; }

int wp_nn_queries_per_block() { return NN_QPB; }
int wp_nn_select_warps() { return NN_SEL_WARPS; }
int wp_nn_hmax() { return NN_HMAX; }

template <int DP>
static cudaError_t launch_dist(bool hist, dim3 grid, cudaStream_t s, const NNArgs& a) {
    const size_t smem = wp_nn_dist_smem_bytes(DP, hist);
    if (hist) {
        cudaFuncSetAttribute(wp_nn_hist_kernel<DP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        wp_nn_hist_kernel<DP><<<grid, NN_THREADS, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(wp_nn_collect_kernel<DP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        wp_nn_collect_kernel<DP><<<grid, NN_THREADS, smem, s>>>(a);
    }
    return cudaGetLastError();
}

// DP: padded dimension, one of 16, 32, 48, 64.  Grid: query blocks x the
// args' entry slices.
cudaError_t wp_launch_nn_dist(int DP, bool hist, cudaStream_t s, const NNArgs& a) {
    const int qblocks = (a.R + NN_QPB - 1) / NN_QPB;
    if (qblocks == 0) return cudaSuccess;
    const dim3 grid(qblocks, a.slices * (hist && a.sub > 1 ? a.sub : 1));
    switch (DP) {
        case 16: return launch_dist<16>(hist, grid, s, a);
        case 32: return launch_dist<32>(hist, grid, s, a);
        case 48: return launch_dist<48>(hist, grid, s, a);
        case 64: return launch_dist<64>(hist, grid, s, a);
        default: return cudaErrorInvalidValue;
    }
}

template <int DP>
static cudaError_t launch_estimate(dim3 grid, cudaStream_t s, const NNArgs& a) {
    const size_t smem = wp_nn_dist_smem_bytes(DP, true);
    cudaFuncSetAttribute(wp_nn_estimate_kernel<DP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    wp_nn_estimate_kernel<DP><<<grid, NN_THREADS, smem, s>>>(a);
    return cudaGetLastError();
}

// The per-query bin origins (a.qbase) from a.sample_n sampled entries.
cudaError_t wp_launch_nn_estimate(int DP, cudaStream_t s, const NNArgs& a) {
    const int qblocks = (a.R + NN_QPB - 1) / NN_QPB;
    if (qblocks == 0) return cudaSuccess;
    const dim3 grid(qblocks);
    switch (DP) {
        case 16: return launch_estimate<16>(grid, s, a);
        case 32: return launch_estimate<32>(grid, s, a);
        case 48: return launch_estimate<48>(grid, s, a);
        case 64: return launch_estimate<64>(grid, s, a);
        default: return cudaErrorInvalidValue;
    }
}

// Reads whose k-th hit fell in the open last bin (the estimate was low):
// listed, their bins moved up by `shift` sixteenths of an octave, to be
// counted again.
__global__ void wp_nn_redo_kernel(NNArgs a, int* list, int* count, int shift) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.R) return;
    const int gq = a.q0 + q;
    const bool beyond = a.tf_d ? !(a.tf_flag[gq] & 1) : a.qcap[gq] >= a.k;
    if (a.qbin[gq] == NN_NB - 1 && beyond) {
        list[atomicAdd(count, 1)] = q;
        a.qbase[gq] += shift;
    }
}

// Zero the per-slice histograms of the listed reads (before a sub-sliced pass).
__global__ void wp_nn_zero_hist_kernel(NNArgs a) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = (long)a.slices * a.R * NN_NB;
    if (i >= n) return;
    const int b = (int)(i % NN_NB);
    const long sq = i / NN_NB;
    const int q = (int)(sq % a.R), s = (int)(sq / a.R);
    a.shist[((long)s * a.R_all + a.q0 + a.slots[q]) * NN_NB + b] = 0u;
}

cudaError_t wp_launch_nn_zero_hist(const NNArgs& a, cudaStream_t s) {
    const long n = (long)a.slices * a.R * NN_NB;
    if (n == 0) return cudaSuccess;
    wp_nn_zero_hist_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t wp_launch_nn_redo(const NNArgs& a, int* list, int* count, int shift, cudaStream_t s) {
    if (a.R == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    wp_nn_redo_kernel<<<(a.R + 255) / 256, 256, 0, s>>>(a, list, count, shift);
    return cudaGetLastError();
}

cudaError_t wp_launch_nn_threshold(cudaStream_t s, const NNArgs& a) {
    if (a.R == 0) return cudaSuccess;
    wp_nn_threshold_kernel<<<(a.R + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t wp_launch_nn_select(int grid, cudaStream_t s, const NNSelectArgs& a) {
    const size_t smem = (sizeof(unsigned long long) * 256 + (sizeof(double) + sizeof(int)) * NN_HMAX) * NN_SEL_WARPS;
    cudaFuncSetAttribute(wp_nn_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    wp_nn_select_kernel<<<grid, NN_SEL_WARPS * 32, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t wp_launch_nn_queries(const double* rads, int R, int TC, int DP, float* out, cudaStream_t s) {
    const long n = (long)R * DP;
    if (n == 0) return cudaSuccess;
    wp_nn_queries_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(rads, R, TC, DP, out);
    return cudaGetLastError();
}

cudaError_t wp_launch_nn_ragged(const int* cand, int h, const int* off, int R, int* out, cudaStream_t s) {
    if (R == 0) return cudaSuccess;
    wp_nn_ragged_kernel<<<R, 128, 0, s>>>(cand, h, off, R, out);
    return cudaGetLastError();
}

// ---- query order ----------------------------------------------------------
// Reads sorted by their first 16 intensities rounded to 0..15 (first one
// most significant), so that the queries of a warp or CTA are alike and skip
// the same far tiles.  Results go back to each read's own index.
__global__ void wp_nn_qkey_kernel(const float* __restrict__ rows, int R, int DP, int TC,
                                  unsigned long long* __restrict__ keys, int* __restrict__ idx) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    unsigned long long k = 0;
    for (int i = 0; i < 16; i++) {
        const float v = i < TC ? rows[(long)r * DP + i] : 0.f;
        const int n = (int)fminf(fmaxf(rintf(v), 0.f), 15.f);
        k = (k << 4) | (unsigned long long)n;
    }
    keys[r] = k;
    idx[r] = r;
}

__global__ void wp_nn_qgather_kernel(const float* __restrict__ rows, const int* __restrict__ perm, int R, int DP,
                                     float* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)R * DP) return;
    const long r = i / DP;
    out[i] = rows[(long)perm[r] * DP + i % DP];
}

size_t wp_nn_sort_temp_bytes(int R) {
    size_t b = 0;
    cub::DoubleBuffer<unsigned long long> k(nullptr, nullptr);
    cub::DoubleBuffer<int> v(nullptr, nullptr);
    cub::DeviceRadixSort::SortPairs(nullptr, b, k, v, R);
    return b;
}

// rows [R][DP] -> sorted [R][DP]; perm[slot] = read.  keys [2R], idx [2R].
cudaError_t wp_launch_nn_sort_queries(const float* rows, int R, int DP, int TC, float* sorted, int* perm,
                                      unsigned long long* keys, int* idx, void* temp, size_t temp_bytes,
                                      cudaStream_t s) {
    if (R == 0) return cudaSuccess;
    wp_nn_qkey_kernel<<<(R + 255) / 256, 256, 0, s>>>(rows, R, DP, TC, keys, idx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cub::DoubleBuffer<unsigned long long> kb(keys, keys + R);
    cub::DoubleBuffer<int> vb(idx, idx + R);
    size_t tb = temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(temp, tb, kb, vb, R, 0, 64, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(perm, vb.Current(), sizeof(int) * R, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    const long n = (long)R * DP;
    wp_nn_qgather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rows, perm, R, DP, sorted);
    return cudaGetLastError();
}
