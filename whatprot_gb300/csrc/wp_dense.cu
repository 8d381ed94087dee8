// wp_dense.cu -- dense warp-per-pair forward pass: the fallback for pairs
// whose pruned boxes exceed the pair engine's per-thread slab.
//
// One warp per (read, peptide) pair; the pair's two state tensors (normal
// and broken-N) are held over the full extents [0, D_c + 1) per channel in
// shared memory, lanes striding over states.  Instead of restricting each
// step to its pruned box, every state is computed and the emission factors
// are zero outside the read's emission box [cmin_t, cmax_t); because dye
// counts never increase this reproduces the reference's pruned result
// exactly (the only leak, the detached-state sum, is dropped by the
// allow-detached flags in the same timesteps as in the reference,
// hmm/step/peptide-emission.cc:218-223).  Same FP32 arithmetic and exact
// power-of-two rescaling as the pair engine.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

#define WP_DENSE_WARPS_MAX 16

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
__device__ void pair_forward(const BatchArgs& a, const SmemModel& H, int r,
                             const DevModel& m, const PeptideRec& pep,
                             const WarpBufs& wb, int S_cap, int lane,
                             float* out_mant, int* out_expo, int* err) {
    const int C = m.C, T = m.T;
    const int W_read = a.W;
    const EmitEntry* __restrict__ rtab = a.tab + (long)r * a.entries;
    const uint8_t* blo = a.lo + (long)r * T * C;
    const uint8_t* bhi = a.hi + (long)r * T * C;
    int Wc[WP_MAX_CHANNELS], st[WP_MAX_CHANNELS];
    int S = 1;
    bool empty = a.flags[r] != 0;
    for (int c = 0; c < C; c++) {
        Wc[c] = pep.D[c] + 1;
        if (pep.D[c] < a.Lsuf[(long)r * T * C + c]) empty = true;  // some L_t > D_c
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
                // largest exponent over [cmin, min(cmax, D + 1)) of channel c
                int km = WP_EXPO_ZERO;
                int n1 = min((int)bhi[t * C + c], Wc[c]);
                for (int n = blo[t * C + c]; n < n1; n++) {
                    EmitEntry en = rtab[(t * C + c) * W_read + n];
                    if (en.mant != 0.0f) km = max(km, en.expo);
                }
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
        pd = a.allow[(long)r * T + t] ? pd * em0 : 0.0f;
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


// Persistent: warps take overflow pairs one at a time.
template <bool HAS_BLOCK>
__global__ void __launch_bounds__(WP_DENSE_WARPS_MAX * 32) wp_dense_kernel(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemModel& M = *reinterpret_cast<SmemModel*>(smem_raw);
    const DevModel& m = *a.model;
    load_smem_model(M, m);
    __syncthreads();
    const int T = m.T, C = m.C;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    unsigned char* wbase = smem_raw + ((sizeof(SmemModel) + 15) & ~(size_t)15);
    size_t wbytes = wp_warp_bytes(T, a.dense_S_cap, C, HAS_BLOCK);
    float* fb = reinterpret_cast<float*>(wbase + wbytes * warp);
    WarpBufs wb;
    size_t slab = (size_t)T * a.dense_S_cap;
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
    wb.coord = reinterpret_cast<uint16_t*>(after + a.dense_S_cap);
    wb.fib = wb.coord + a.dense_S_cap;
    const int count = *a.ovf_count;
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(a.ovf_head, 1);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= count) break;
        const int2 rg = a.ovf[idx];
        int vmax;
        const PeptideRec& pep = a.peps[slot_pep(a, rg.x, item_slot(a, rg, &vmax))];
        float mant;
        int ex;
        pair_forward<HAS_BLOCK>(a, M, rg.x, m, pep, wb, a.dense_S_cap, lane, &mant, &ex, a.err);
        if (lane == 0) {
            a.res_mant[rg.y] = mant;
            a.res_expo[rg.y] = ex;
        }
        __syncwarp();
    }
}

size_t wp_dense_smem_bytes(int T, int S_cap, int C, bool has_block, int warps) {
    return ((sizeof(SmemModel) + 15) & ~(size_t)15) + wp_warp_bytes(T, S_cap, C, has_block) * warps;
}

// Persistent grid of one CTA per SM (overflow pairs are few).
cudaError_t wp_launch_dense(bool has_block, int threads, size_t smem, cudaStream_t stream,
                            const BatchArgs& a) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    if (has_block) {
        e = cudaFuncSetAttribute(wp_dense_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        wp_dense_kernel<true><<<sms, threads, smem, stream>>>(a);
    } else {
        e = cudaFuncSetAttribute(wp_dense_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        wp_dense_kernel<false><<<sms, threads, smem, stream>>>(a);
    }
    return cudaGetLastError();
}
