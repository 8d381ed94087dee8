// wp_engine.cu -- the pair engine: one thread per (read, peptide) pair.
//
// Each thread runs the reference's pruned step chain for its pair
// (hmm/hmm/peptide-hmm.cc:40-61: initial block, dud per channel, emission 0,
// then per timestep cyclic block, detach, bleach per channel, Edman,
// emission) over exactly the boxes the reference's prune passes leave
// (see wp_prep.cu), so the work per pair is the reference's visited-state
// work.  FP32 arithmetic; after every emission the state is rescaled by an
// exact power of two and the exponent is carried as an integer, so nothing
// underflows and no FP64 is needed in the loop.
//
// State storage.  A pair's state is one dense box per step (row-major over
// Edman count e and the dye count of each channel, anchored at the box's
// lower corner).  Each thread owns a slab of shared memory holding two such
// boxes (ping-pong) plus its per-channel emission factors; slabs are
// interleaved across the CTA's threads (element k of thread i at
// k * blockDim.x + i) so every access of a warp hits 32 distinct banks
// whatever the index.  A pair whose largest box does not fit its slab is
// handed to the overflow list (wp_dense.cu).
//
// With blocking (p_initial_block or p_cyclic_block nonzero) each state holds
// the normal and the broken-N value as a float2.
#include <cuda_runtime.h>
#include <stdint.h>

#include "wp_common.cuh"

#define WP_ENGINE_THREADS 256

template <bool HB>
struct StateOf;
template <>
struct StateOf<false> {
    using V = float;
};
template <>
struct StateOf<true> {
    using V = float2;
};

__device__ __forceinline__ float vzero(float) { return 0.0f; }
__device__ __forceinline__ float2 vzero(float2) { return make_float2(0.0f, 0.0f); }
__device__ __forceinline__ float vfma(float k, float v, float acc) { return fmaf(k, v, acc); }
__device__ __forceinline__ float2 vfma(float k, float2 v, float2 acc) {
    return make_float2(fmaf(k, v.x, acc.x), fmaf(k, v.y, acc.y));
}
__device__ __forceinline__ float vmul(float k, float v) { return k * v; }
__device__ __forceinline__ float2 vmul(float k, float2 v) { return make_float2(k * v.x, k * v.y); }
__device__ __forceinline__ float vtotal(float v) { return v; }
__device__ __forceinline__ float vtotal(float2 v) { return v.x + v.y; }

// Box of one step: per-channel [lo, lo + w).
template <int C>
struct Box {
    int lo[C];
    int w[C];
    __device__ __forceinline__ int vol() const {
        int v = 1;
#pragma unroll
        for (int c = 0; c < C; c++) v *= w[c];
        return v;
    }
};

// Binomial transition along channel c (BinomialTransition::forward,
// hmm/step/binomial-transition.cc:104-136) from box `in` to box `out`, which
// differ only on channel c, over E Edman slices:
//   out[to] = sum_{from >= to, from in box} prob(from, to) * in[from].
template <int C, class V>
__device__ __forceinline__ void binomial_boxes(const V* __restrict__ src, V* __restrict__ dst,
                                               int stride, int E, const Box<C>& in,
                                               const Box<C>& out, int ch,
                                               const float* __restrict__ tab) {
    int outer = E, inner = 1, win = 1, wout = 1, from0 = 0, to0 = 0;
#pragma unroll
    for (int c = 0; c < C; c++) {
        if (c < ch) outer *= in.w[c];
        if (c > ch) inner *= in.w[c];
        if (c == ch) {
            win = in.w[c];
            wout = out.w[c];
            from0 = in.lo[c];
            to0 = out.lo[c];
        }
    }
    for (int o = 0; o < outer; o++) {
        for (int k2 = 0; k2 < wout; k2++) {
            const int to = to0 + k2;
            const int kmin = max(0, to - from0);
            const V* s = src + (o * win) * inner * stride;
            V* d = dst + ((o * wout + k2) * inner) * stride;
            for (int i = 0; i < inner; i++) {
                V acc = vzero(V());
                for (int k = kmin; k < win; k++) {
                    const int from = from0 + k;
                    acc = vfma(tab[from * (from + 1) / 2 + to], s[(k * inner + i) * stride], acc);
                }
                d[i * stride] = acc;
            }
        }
    }
}

// Runs one pair.  Returns 1 when its boxes exceed the slab (nothing
// written), else 0 with P = *mant * 2^*expo (mant == 0: P == 0).
template <int C, bool HB>
__device__ int engine_pair(const BatchArgs& a, const SmemModel& M, int r,
                           const PeptideRec& pep, typename StateOf<HB>::V* slab,
                           float* scr, int stride, int half, float* out_mant, int* out_expo) {
    using V = typename StateOf<HB>::V;
    const DevModel& m = *a.model;
    const int T = m.T;
    const uint8_t* Ls = a.Lsuf + (long)r * T * C;
    const uint8_t* Up = a.Upre + (long)r * T * C;
    const uint8_t* allow = a.allow + (long)r * T;
    const EmitEntry* tab = a.tab + (long)r * a.entries;
    int D1[C];
#pragma unroll
    for (int c = 0; c < C; c++) D1[c] = pep.D[c] + 1;

    // Boxes per timestep: Nx_t = [L_t, U_t) (emission), Bt_t = [L_t,
    // min(U_t + 1, U_{t-1})) (bleach output / Edman input).  First pass:
    // the largest box any step of this pair uses.
    int need;
    {
        int v0 = 1, vmax = 0;
#pragma unroll
        for (int c = 0; c < C; c++) v0 *= D1[c] - Ls[c];
        vmax = v0;
        for (int t = 1; t < T; t++) {
            int vp = t, vb = t, vn = t + 1;
            int mix[C];
#pragma unroll
            for (int c = 0; c < C; c++) {
                int lp = Ls[(t - 1) * C + c], up = min((int)Up[(t - 1) * C + c], D1[c]);
                int ln = Ls[t * C + c], un = min((int)Up[t * C + c], D1[c]);
                int bu = min(un + 1, up);
                vp *= up - lp;
                vb *= bu - ln;
                vn *= un - ln;
                mix[c] = (bu - ln) > (up - lp) ? (bu - ln) : (up - lp);
            }
            int vm = t;
#pragma unroll
            for (int c = 0; c < C; c++) vm *= mix[c];
            vmax = max(vmax, max(max(vp, vb), max(vn, vm)));
        }
        need = vmax;
    }
    if (need > half) return 1;

    V* cur = slab;
    V* nxt = slab + half * stride;
    auto swap_bufs = [&]() {
        V* tmp = cur;
        cur = nxt;
        nxt = tmp;
    };

    // ---- t = 0: start state (0, D) (peptide-state-vector.cc:38-40) in the
    // box [L_0, D + 1), initial block, duds.
    Box<C> bx;
#pragma unroll
    for (int c = 0; c < C; c++) {
        bx.lo[c] = Ls[c];
        bx.w[c] = D1[c] - Ls[c];
    }
    {
        int v = bx.vol();
        for (int i = 0; i < v - 1; i++) cur[i * stride] = vzero(V());
        V start = vzero(V());
        if constexpr (HB) {
            start = make_float2(1.0f - m.p_ib, m.p_ib);  // block-transition.cc:33-62
        } else {
            start = 1.0f;
        }
        cur[(v - 1) * stride] = start;
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
        Box<C> ob = bx;
        int u0 = min((int)Up[c], D1[c]);
        ob.w[c] = u0 - bx.lo[c];
        binomial_boxes<C, V>(cur, nxt, stride, 1, bx, ob, c, M.dud[c]);
        swap_bufs();
        bx = ob;
    }

    int expo = 0;           // the true state is the stored state times 2^expo
    float pd = 0.0f;        // detached state, in the rescaled frame
    int k_prev = 0;         // exponent removed at the last rescale
    float fac_prev = 1.0f;  // (1 - p_detach) pending from the last timestep
    for (int t = 0; t < T; t++) {
        Box<C> nx;  // emission box [L_t, U_t)
#pragma unroll
        for (int c = 0; c < C; c++) {
            nx.lo[c] = Ls[t * C + c];
            nx.w[c] = min((int)Up[t * C + c], D1[c]) - nx.lo[c];
        }
        if (t > 0) {
            // Cyclic block (block-transition.cc:33-62) over e < t and the
            // previous emission box.
            if constexpr (HB) {
                if (m.p_cb != 0.0f) {
                    int n = t * bx.vol();
                    for (int i = 0; i < n; i++) {
                        float2 s = cur[i * stride];
                        cur[i * stride] = make_float2((1.0f - m.p_cb) * s.x, s.y + m.p_cb * s.x);
                    }
                }
            }
            // Detach (detach-transition.cc:36-68) was folded into the last
            // rescale: pd already holds it, fac_prev carries (1 - p).
            // Bleach per channel: channel c moves from the previous box to
            // [L_t, min(U_t + 1, U_{t-1})).
#pragma unroll
            for (int c = 0; c < C; c++) {
                Box<C> ob = bx;
                int bu = min(nx.lo[c] + nx.w[c] + 1, bx.lo[c] + bx.w[c]);
                ob.lo[c] = nx.lo[c];
                ob.w[c] = bu - nx.lo[c];
                binomial_boxes<C, V>(cur, nxt, stride, t, bx, ob, c, M.bleach[c]);
                swap_bufs();
                bx = ob;
            }
            // Edman (edman-transition.cc:62-162) as a gather from slices
            // e-1 (success) and e (failure) into the emission box.
            {
                const float pf = m.pf, qf = 1.0f - m.pf;
                int stb[C], stn[C];
                int vb = 1, vn = 1;
#pragma unroll
                for (int c = C - 1; c >= 0; c--) {
                    stb[c] = vb;
                    stn[c] = vn;
                    vb *= bx.w[c];
                    vn *= nx.w[c];
                }
                for (int e = 0; e <= t; e++) {
                    int dc = e >= 1 ? pep.dye[e - 1] : -1;
                    float tot = e >= 1 ? (float)pep.tot[e - 1] : 1.0f;
                    // Select the removal channel's box terms once per slice.
                    int d_lo = 0, d_wb = 0, d_st = 0;
#pragma unroll
                    for (int c = 0; c < C; c++)
                        if (c == dc) {
                            d_lo = nx.lo[c];
                            d_wb = bx.w[c];
                            d_st = stb[c];
                        }
                    int jc[C];
#pragma unroll
                    for (int c = 0; c < C; c++) jc[c] = 0;
                    int ib = 0;
                    for (int j = 0; j < vn; j++) {
                        V v = vzero(V());
                        if (e < t) {
                            V f = cur[(e * vb + ib) * stride];
                            if constexpr (HB) {
                                v = make_float2(pf * f.x, f.y);  // broken-N copied unchanged
                            } else {
                                v = pf * f;
                            }
                        }
                        if (e >= 1) {
                            float xin;
                            if constexpr (HB) {
                                xin = cur[((e - 1) * vb + ib) * stride].x;
                            } else {
                                xin = cur[((e - 1) * vb + ib) * stride];
                            }
                            float add;
                            if (dc < 0) {
                                add = qf * xin;
                            } else {
                                int jd = 0;
#pragma unroll
                                for (int c = 0; c < C; c++)
                                    if (c == dc) jd = jc[c];
                                const int nc = d_lo + jd;
                                add = 0.0f;
                                if ((float)nc < tot) add = qf * (1.0f - (float)nc / tot) * xin;
                                if (jd + 1 < d_wb) {
                                    float xr;
                                    if constexpr (HB) {
                                        xr = cur[((e - 1) * vb + ib + d_st) * stride].x;
                                    } else {
                                        xr = cur[((e - 1) * vb + ib + d_st) * stride];
                                    }
                                    add = fmaf(qf * ((float)(nc + 1) / tot), xr, add);
                                }
                            }
                            if constexpr (HB) {
                                v.x += add;
                            } else {
                                v += add;
                            }
                        }
                        nxt[(e * vn + j) * stride] = v;
                        // advance the multi-index over the emission box
#pragma unroll
                        for (int c = C - 1; c >= 0; c--) {
                            jc[c]++;
                            ib += stb[c];
                            if (jc[c] < nx.w[c]) break;
                            ib -= stb[c] * nx.w[c];
                            jc[c] = 0;
                        }
                    }
                }
                swap_bufs();
                bx = nx;
            }
        }
        // ---- Emission t (peptide-emission.cc:212-243).  Per-channel factors
        // normalised by their largest exponent over the pair's box, stored
        // in the scratch; the pending rescale is folded into the multiplier.
        int kmax = 0;
        bool dead = false;
        int goff[C];
        {
            int off = 0;
#pragma unroll
            for (int c = 0; c < C; c++) {
                goff[c] = off;
                off += nx.w[c];
            }
        }
        if (!m.interacting) {
#pragma unroll
            for (int c = 0; c < C; c++) {
                const EmitEntry* row = tab + (t * C + c) * a.W + nx.lo[c];
                int km = WP_EXPO_ZERO;
                for (int k = 0; k < nx.w[c]; k++)
                    if (row[k].mant != 0.0f) km = max(km, row[k].expo);
                if (km == WP_EXPO_ZERO) dead = true;
                kmax += km;
                for (int k = 0; k < nx.w[c]; k++) {
                    EmitEntry en = row[k];
                    scr[(goff[c] + k) * stride] =
                            en.mant != 0.0f ? en.mant * exp2i(max(en.expo - km, -200)) : 0.0f;
                }
            }
        }
        if (dead) {
            *out_mant = 0.0f;
            *out_expo = 0;
            return 0;
        }
        const float sfac = fac_prev * exp2i(-k_prev);
        float part = 0.0f;
        float em0 = 0.0f;
        const int vn = nx.vol();
        if (!m.interacting) {
            // emission factor of state n is prod_c g_c[n_c - L_t]
            if (allow[t]) {
                em0 = 1.0f;
#pragma unroll
                for (int c = 0; c < C; c++) em0 *= scr[goff[c] * stride];
            }
            int jc[C];
#pragma unroll
            for (int c = 0; c < C; c++) jc[c] = 0;
            for (int j = 0; j < vn; j++) {
                float w = sfac;
#pragma unroll
                for (int c = 0; c < C; c++) w *= scr[(goff[c] + jc[c]) * stride];
                for (int e = 0; e <= t; e++) {
                    V s = vmul(w, cur[(e * vn + j) * stride]);
                    cur[(e * vn + j) * stride] = s;
                    part += vtotal(s);
                }
#pragma unroll
                for (int c = C - 1; c >= 0; c--) {
                    jc[c]++;
                    if (jc[c] < nx.w[c]) break;
                    jc[c] = 0;
                }
            }
        } else {
            // Interacting channels: one factor per dye-count vector.
            const int G = wp_ipow(a.W, C);
            int km = WP_EXPO_ZERO;
            int jc[C];
#pragma unroll
            for (int c = 0; c < C; c++) jc[c] = 0;
            for (int j = 0; j < vn; j++) {
                int gi = 0;
#pragma unroll
                for (int c = 0; c < C; c++) gi = gi * a.W + nx.lo[c] + jc[c];
                EmitEntry en = tab[t * G + gi];
                if (en.mant != 0.0f) km = max(km, en.expo);
#pragma unroll
                for (int c = C - 1; c >= 0; c--) {
                    jc[c]++;
                    if (jc[c] < nx.w[c]) break;
                    jc[c] = 0;
                }
            }
            if (km == WP_EXPO_ZERO) {
                *out_mant = 0.0f;
                *out_expo = 0;
                return 0;
            }
            kmax = km;
            if (allow[t]) {
                EmitEntry en = tab[t * G];
                em0 = en.mant != 0.0f ? en.mant * exp2i(max(en.expo - km, -200)) : 0.0f;
            }
            for (int j = 0; j < vn; j++) {
                int gi = 0;
#pragma unroll
                for (int c = 0; c < C; c++) gi = gi * a.W + nx.lo[c] + jc[c];
                EmitEntry en = tab[t * G + gi];
                float w = en.mant != 0.0f ? sfac * (en.mant * exp2i(max(en.expo - km, -200))) : 0.0f;
                for (int e = 0; e <= t; e++) {
                    V s = vmul(w, cur[(e * vn + j) * stride]);
                    cur[(e * vn + j) * stride] = s;
                    part += vtotal(s);
                }
#pragma unroll
                for (int c = C - 1; c >= 0; c--) {
                    jc[c]++;
                    if (jc[c] < nx.w[c]) break;
                    jc[c] = 0;
                }
            }
        }
        // Detached state: kept only while the box includes zero
        // (peptide-emission.cc:218-223).
        pd = allow[t] ? pd * em0 : 0.0f;
        expo += kmax;
        const float tot = part + pd;
        if (!(tot > 0.0f) || !isfinite(tot)) {
            *out_mant = 0.0f;
            *out_expo = 0;
            return 0;
        }
        int k;
        const float fm = frexpf(tot, &k);
        if (t == T - 1) {
            *out_mant = fm;
            *out_expo = expo + k;
            return 0;
        }
        expo += k;
        const float f = exp2i(-k);
        // Detach of the next timestep in the rescaled frame
        // (detach-transition.cc:36-68): p_detached += p * sum of the states.
        pd = (pd + M.p_det[t] * part) * f;
        k_prev = k;
        fac_prev = 1.0f - M.p_det[t];
    }
    *out_mant = 0.0f;
    *out_expo = 0;
    return 0;
}

// Persistent: each warp takes 32 consecutive work items at a time.
// Lists one engine pass reads and spills to.
struct EngineLists {
    const int2* in;
    const int* in_count;
    int* in_head;
    int2* out;
    int* out_count;
    int slab_half;
    int scr_floats;
    int spill_error;  // nonzero: nothing downstream takes spills; flag err
};

template <int C, bool HB>
__global__ void __launch_bounds__(WP_ENGINE_THREADS) wp_engine_kernel(BatchArgs a, EngineLists L) {
    using V = typename StateOf<HB>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemModel& M = *reinterpret_cast<SmemModel*>(smem_raw);
    load_smem_model(M, *a.model);
    __syncthreads();
    const int nt = blockDim.x;
    V* slab_region = reinterpret_cast<V*>(smem_raw + ((sizeof(SmemModel) + 15) & ~(size_t)15));
    float* scr_region = reinterpret_cast<float*>(slab_region + (size_t)2 * L.slab_half * nt);
    V* slab = slab_region + threadIdx.x;
    float* scr = scr_region + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int count = *L.in_count;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(L.in_head, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= count) break;
        const int w = base + lane;
        if (w < count) {
            const int2 rg = L.in[w];
            const int p = slot_pep(a, rg.x, rg.y);
            float mant;
            int ex;
            int ov = engine_pair<C, HB>(a, M, rg.x, a.peps[p], slab, scr, nt, L.slab_half, &mant, &ex);
            if (ov) {
                if (L.spill_error) {
                    atomicExch(a.err, 2);
                    a.res_mant[rg.y] = 0.0f;
                    a.res_expo[rg.y] = 0;
                } else {
                    int q = atomicAdd(L.out_count, 1);
                    L.out[q] = rg;
                }
            } else {
                a.res_mant[rg.y] = mant;
                a.res_expo[rg.y] = ex;
            }
        }
    }
}

size_t wp_engine_smem_bytes(int slab_half, int scr_floats, bool has_block, int threads) {
    size_t elem = has_block ? sizeof(float2) : sizeof(float);
    return ((sizeof(SmemModel) + 15) & ~(size_t)15) + (size_t)2 * slab_half * threads * elem +
           (size_t)scr_floats * threads * sizeof(float);
}

template <int C, bool HB>
static cudaError_t launch_engine(int threads, size_t smem, cudaStream_t s, const BatchArgs& a,
                                 const EngineLists& L, int* grid_out) {
    cudaError_t e = cudaFuncSetAttribute(wp_engine_kernel<C, HB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wp_engine_kernel<C, HB>, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int grid = sms * per_sm;
    if (grid_out) *grid_out = grid;
    wp_engine_kernel<C, HB><<<grid, threads, smem, s>>>(a, L);
    return cudaGetLastError();
}

// One engine pass over a work list (persistent grid: SMs x resident CTAs).
cudaError_t wp_launch_engine(int C, bool has_block, int threads, size_t smem, cudaStream_t s,
                             const BatchArgs& a, const int2* in, const int* in_count, int* in_head,
                             int2* out, int* out_count, int slab_half, int scr_floats,
                             int spill_error, int* grid_out) {
    EngineLists L{in, in_count, in_head, out, out_count, slab_half, scr_floats, spill_error};
    switch (C * 2 + (has_block ? 1 : 0)) {
        case 2: return launch_engine<1, false>(threads, smem, s, a, L, grid_out);
        case 3: return launch_engine<1, true>(threads, smem, s, a, L, grid_out);
        case 4: return launch_engine<2, false>(threads, smem, s, a, L, grid_out);
        case 5: return launch_engine<2, true>(threads, smem, s, a, L, grid_out);
        case 6: return launch_engine<3, false>(threads, smem, s, a, L, grid_out);
        case 7: return launch_engine<3, true>(threads, smem, s, a, L, grid_out);
        case 8: return launch_engine<4, false>(threads, smem, s, a, L, grid_out);
        case 9: return launch_engine<4, true>(threads, smem, s, a, L, grid_out);
        default: return cudaErrorInvalidValue;
    }
}

int wp_engine_max_threads() { return WP_ENGINE_THREADS; }
