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
// boxes (ping-pong); slabs are interleaved across the CTA's threads (element
// k of thread i at k * blockDim.x + i) so every access of a warp hits 32
// distinct banks whatever the index.  The compaction (wp_prep.cu) routes
// each pair to the first pass whose slab holds its largest box and leaves
// that box's size with the pair (BatchArgs::pair_info, or its result slot);
// a pass checks it against its slab before any write and hands a pair that
// does not fit to the next pass's list.
//
// Boxes are kept packed, one byte per channel in a 32-bit word (lower
// corner) and another (width), so that the per-channel loops need no
// unrolling; the binomial step is one out-of-line routine shared by the dud
// and bleach steps, and the rarely taken paths (wide boxes, interacting
// channels) are out of line too.  This keeps the timestep loop small enough
// for the instruction cache.
//
// Two shortcuts follow from the box statistics of real workloads, where
// most timesteps of most pairs have a one-state emission box: a bleach step
// along a channel that is one wide on both sides is a single coefficient,
// carried to the next emission multiply instead of a pass over the state
// (checked for all channels at once with word operations); and Edman and
// emission run as one loop, state outer and Edman slice inner (two slices
// at a time), for every emission box at most 4 wide per channel, one-state
// boxes included.  The start state goes through the duds as one product per
// state, written straight into the first emission box.  Edman coefficients
// come from per-CTA tables indexed by (dye count of the state, remaining
// dyes of the cut channel); each position's (cut channel, remaining dyes)
// is a code byte in the thread's slice of shared memory, and one byte
// permute of the state's packed counts picks the count it needs.
// All lanes of a warp process the same timestep together (lanes are pairs
// of one read), so a warp pays for every path any of its lanes takes in a
// timestep; the number of distinct paths is kept small for that reason.  A
// separate one-state path (cheaper per lane) cost more than it saved, as
// warps whose lanes mixed one-state and wider boxes ran both paths.
//
// With blocking (p_initial_block or p_cyclic_block nonzero) each state holds
// the normal and the broken-N value as a float2.
#include <cuda_runtime.h>
#include <stdint.h>

#include "wp_common.cuh"

#define WP_ENGINE_THREADS 256
#define WP_ENGINE_CODES 16  // Edman code bytes per thread (positions 0..15)

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

// Packed box: byte c of lo / w is channel c's lower corner / width.
struct PBox {
    uint32_t lo;
    uint32_t w;
};
__device__ __forceinline__ int bget(uint32_t v, int c) { return (int)((v >> (8 * c)) & 0xffu); }
// prmt.b32 in its default mode: byte n of the result is the byte of {y, x}
// (x: bytes 0-3, y: 4-7) that nibble n of s selects, its sign replicated
// where the nibble's bit 3 is set.
__device__ __forceinline__ uint32_t prmt(uint32_t x, uint32_t y, uint32_t s) {
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(x), "r"(y), "r"(s));
    return d;
}
__device__ __forceinline__ uint32_t bset(uint32_t v, int c, int x) {
    return (v & ~(0xffu << (8 * c))) | ((uint32_t)x << (8 * c));
}
// The bytes of a packed word that hold channels.
template <int C>
__device__ __forceinline__ uint32_t chan_mask() {
    return C >= 4 ? 0xffffffffu : (1u << (8 * C)) - 1u;
}

template <int C>
__device__ __forceinline__ int bvol(uint32_t w) {
    int v = 1;
#pragma unroll
    for (int c = 0; c < C; c++) v *= bget(w, c);
    return v;
}

// Binomial transition along channel ch (BinomialTransition::forward,
// hmm/step/binomial-transition.cc:104-136) from box `in` to the box with
// channel ch moved to [to0, to0 + wout), over E Edman slices:
//   out[to] = sum_{from >= to, from in box} prob(from, to) * in[from].
template <int C, class V>
__device__ __noinline__ void binomial_step(const V* __restrict__ src, V* __restrict__ dst, int stride,
                                           int E, PBox in, int ch, int to0, int wout,
                                           const float* __restrict__ tab) {
    int outer = E, inner = 1;
#pragma unroll
    for (int c = 0; c < C; c++) {
        const int w = bget(in.w, c);
        if (c < ch) outer *= w;
        if (c > ch) inner *= w;
    }
    const int win = bget(in.w, ch), from0 = bget(in.lo, ch);
    const int sk = inner * stride;
    if (win <= 3 && wout <= 3) {
        // The coefficients prob(from0 + k -> to0 + k2) in registers; each
        // input column (its up to 3 states along ch) is loaded once and
        // gives all the column's outputs.
        float cf[3][3];
        // prob(from0 + k -> to0) sits at rb[k]; prob(from0 + k -> to0 + k2)
        // at rb[k] + k2 (triangular rows), nonzero only for from >= to.
        const int rb0 = from0 * (from0 + 1) / 2 + to0;
        const int rb[3] = {rb0, rb0 + from0 + 1, rb0 + 2 * from0 + 3};
        const int d = from0 - to0;
#pragma unroll
        for (int k2 = 0; k2 < 3; k2++)
#pragma unroll
            for (int k = 0; k < 3; k++)
                cf[k2][k] = (k < win && k2 < wout && d + k - k2 >= 0) ? tab[rb[k] + k2] : 0.0f;
        // the outer x inner columns as one sequence, two at a time
        // (independent loads and chains)
        const int n = outer * inner;
        const int ostep_in = win * sk - inner * stride, ostep_out = wout * sk - inner * stride;
        const V* si = src;
        V* di = dst;
        int i = 0;
        auto next = [&]() {
            si += stride;
            di += stride;
            if (++i == inner) {
                i = 0;
                si += ostep_in;
                di += ostep_out;
            }
        };
        int q = 0;
        for (; q + 1 < n; q += 2) {
            const V* sa = si;
            V* da = di;
            next();
            const V* sb = si;
            V* db = di;
            next();
            const V a0 = sa[0], b0 = sb[0];
            const V a1 = win > 1 ? sa[sk] : vzero(V()), b1 = win > 1 ? sb[sk] : vzero(V());
            const V a2 = win > 2 ? sa[2 * sk] : vzero(V()), b2 = win > 2 ? sb[2 * sk] : vzero(V());
#pragma unroll
            for (int k2 = 0; k2 < 3; k2++)
                if (k2 < wout) {
                    da[k2 * sk] = vfma(cf[k2][2], a2, vfma(cf[k2][1], a1, vmul(cf[k2][0], a0)));
                    db[k2 * sk] = vfma(cf[k2][2], b2, vfma(cf[k2][1], b1, vmul(cf[k2][0], b0)));
                }
        }
        if (q < n) {
            const V x0 = si[0];
            const V x1 = win > 1 ? si[sk] : vzero(V());
            const V x2 = win > 2 ? si[2 * sk] : vzero(V());
#pragma unroll
            for (int k2 = 0; k2 < 3; k2++)
                if (k2 < wout) di[k2 * sk] = vfma(cf[k2][2], x2, vfma(cf[k2][1], x1, vmul(cf[k2][0], x0)));
        }
        return;
    }
    if (win <= 4) {
        // Coefficients depend on (to, from) only: load them once per output
        // row, then one predicated dot product per column.
        for (int k2 = 0; k2 < wout; k2++) {
            const int to = to0 + k2;
            float cf[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int from = from0 + k;
                cf[k] = (k < win && from >= to) ? tab[from * (from + 1) / 2 + to] : 0.0f;
            }
            // the columns as one sequence, two at a time (as above)
            const int n = outer * inner;
            const int ostep_in = win * sk - inner * stride, ostep_out = wout * sk - inner * stride;
            const V* si = src;
            V* di = dst + k2 * sk;
            int i = 0;
            auto next = [&]() {
                si += stride;
                di += stride;
                if (++i == inner) {
                    i = 0;
                    si += ostep_in;
                    di += ostep_out;
                }
            };
            auto dot = [&](const V* x) {
                V acc = vmul(cf[0], x[0]);
                if (win > 1) acc = vfma(cf[1], x[sk], acc);
                if (win > 2) acc = vfma(cf[2], x[2 * sk], acc);
                if (win > 3) acc = vfma(cf[3], x[3 * sk], acc);
                return acc;
            };
            int q = 0;
            for (; q + 1 < n; q += 2) {
                const V* sa = si;
                V* da = di;
                next();
                const V* sb = si;
                V* db = di;
                next();
                const V ra = dot(sa), rb = dot(sb);
                *da = ra;
                *db = rb;
            }
            if (q < n) *di = dot(si);
        }
        return;
    }
    for (int o = 0; o < outer; o++) {
        for (int k2 = 0; k2 < wout; k2++) {
            const int to = to0 + k2;
            const int kmin = max(0, to - from0);
            const V* s = src + o * win * sk;
            V* d = dst + (o * wout + k2) * sk;
            for (int i = 0; i < inner; i++) {
                V acc = vzero(V());
                for (int k = kmin; k < win; k++) {
                    const int from = from0 + k;
                    acc = vfma(tab[from * (from + 1) / 2 + to], s[k * sk + i * stride], acc);
                }
                d[i * stride] = acc;
            }
        }
    }
}

// Emission multiply for boxes with a channel wider than 4, or interacting
// channels: the factor of each state read from the table.  Returns the sum
// of the multiplied states; *kmax_out receives the normalising exponent
// (WP_EXPO_ZERO: every factor is zero), *em0 the factor of the all-zero
// state (unscaled by the pending rescale).
template <int C, class V>
__device__ __noinline__ float emission_table(V* cur, int stride, int t, PBox nx, int W,
                                             const EmitEntry* __restrict__ tab, bool interacting,
                                             float fac_prev, int k_prev, int* kmax_out, float* em0) {
    const int vn = bvol<C>(nx.w);
    const int G = interacting ? wp_ipow(W, C) : 0;
    int jc[C];
    // pass 1: normalising exponent over the box
    int kmax = 0;
    if (!interacting) {
#pragma unroll
        for (int c = 0; c < C; c++) {
            const EmitEntry* row = tab + (t * C + c) * W + bget(nx.lo, c);
            int km = WP_EXPO_ZERO;
            for (int k = 0; k < bget(nx.w, c); k++)
                if (row[k].mant != 0.0f) km = max(km, row[k].expo);
            if (km == WP_EXPO_ZERO) {
                *kmax_out = WP_EXPO_ZERO;
                return 0.0f;
            }
            kmax += km;
        }
    } else {
        int km = WP_EXPO_ZERO;
#pragma unroll
        for (int c = 0; c < C; c++) jc[c] = 0;
        for (int j = 0; j < vn; j++) {
            int gi = 0;
#pragma unroll
            for (int c = 0; c < C; c++) gi = gi * W + bget(nx.lo, c) + jc[c];
            EmitEntry en = tab[t * G + gi];
            if (en.mant != 0.0f) km = max(km, en.expo);
#pragma unroll
            for (int c = C - 1; c >= 0; c--) {
                if (++jc[c] < bget(nx.w, c)) break;
                jc[c] = 0;
            }
        }
        if (km == WP_EXPO_ZERO) {
            *kmax_out = WP_EXPO_ZERO;
            return 0.0f;
        }
        kmax = km;
    }
    *kmax_out = kmax;
    // factor of the all-zero state (only used when the box starts at zero)
    {
        float mm = 1.0f;
        int ks = 0;
        if (!interacting) {
#pragma unroll
            for (int c = 0; c < C; c++) {
                EmitEntry en = tab[(t * C + c) * W];
                mm *= en.mant;
                ks += en.expo;
            }
        } else {
            EmitEntry en = tab[t * G];
            mm = en.mant;
            ks = en.expo;
        }
        *em0 = mm != 0.0f ? mm * exp2i(max(ks - kmax, -200)) : 0.0f;
    }
    // pass 2: multiply
    float part = 0.0f;
#pragma unroll
    for (int c = 0; c < C; c++) jc[c] = 0;
    for (int j = 0; j < vn; j++) {
        float mm = fac_prev;
        int ks = 0;
        if (!interacting) {
#pragma unroll
            for (int c = 0; c < C; c++) {
                EmitEntry en = tab[(t * C + c) * W + bget(nx.lo, c) + jc[c]];
                mm *= en.mant;
                ks += en.expo;
            }
        } else {
            int gi = 0;
#pragma unroll
            for (int c = 0; c < C; c++) gi = gi * W + bget(nx.lo, c) + jc[c];
            EmitEntry en = tab[t * G + gi];
            mm *= en.mant;
            ks = en.expo;
        }
        const float w = mm != 0.0f ? mm * exp2i(max(ks - kmax - k_prev, -200)) : 0.0f;
        for (int e = 0; e <= t; e++) {
            V s = vmul(w, cur[(e * vn + j) * stride]);
            cur[(e * vn + j) * stride] = s;
            part += vtotal(s);
        }
#pragma unroll
        for (int c = C - 1; c >= 0; c--) {
            if (++jc[c] < bget(nx.w, c)) break;
            jc[c] = 0;
        }
    }
    return part;
}

// Edman (edman-transition.cc:62-162) as a gather from slices e-1 (success)
// and e (failure) of the bleached box bx (E = t slices in cur) into the
// emission box nx (t + 1 slices in nxt); both boxes share the lower corner
// L_t.  Out of line: a quarter of the timesteps take it, and the one-state
// path's code stays compact in the instruction cache.
template <int C, bool HB>
__device__ __noinline__ void edman_gather(const typename StateOf<HB>::V* __restrict__ cur,
                                          typename StateOf<HB>::V* __restrict__ nxt, int stride, int t, PBox bx,
                                          PBox nx, bool pk, uint64_t dye_pk, uint64_t tot_pk,
                                          const PeptideRec& pep, const float* __restrict__ edx,
                                          const float* __restrict__ edy, float pf) {
    using V = typename StateOf<HB>::V;
    const float qf = 1.0f - pf;
    int stb[C];
    int vb = 1;
#pragma unroll
    for (int c = C - 1; c >= 0; c--) {
        stb[c] = vb;
        vb *= bget(bx.w, c);
    }
    const int vn = bvol<C>(nx.w);
    for (int e = 0; e <= t; e++) {
        int dc = -1, tot_i = 1;
        if (e >= 1) {
            if (pk) {
                dc = (int)((dye_pk >> (4 * (e - 1))) & 15) - 1;
                tot_i = (int)((tot_pk >> (4 * (e - 1))) & 15);
            } else {
                dc = pep.dye[e - 1];
                tot_i = pep.tot[e - 1];
            }
        }
        // Edman coefficients of this slice: column DyeTrack(e - 1, dc)
        int d_lo = 0, d_wb = 0, d_st = 0;
#pragma unroll
        for (int c = 0; c < C; c++)
            if (c == dc) {
                d_lo = bget(nx.lo, c);
                d_wb = bget(bx.w, c);
                d_st = stb[c];
            }
        int jc[C];
#pragma unroll
        for (int c = 0; c < C; c++) jc[c] = 0;
        int ib = 0;
        const V* fail_row = cur + e * vb * stride;
        const V* succ_row = cur + (e - 1) * vb * stride;
        V* out_row = nxt + e * vn * stride;
        for (int j = 0; j < vn; j++) {
            V v = vzero(V());
            if (e < t) {
                const V f = fail_row[ib * stride];
                if constexpr (HB) {
                    v = make_float2(pf * f.x, f.y);  // broken-N copied unchanged
                } else {
                    v = pf * f;
                }
            }
            if (e >= 1) {
                float xin;
                if constexpr (HB) {
                    xin = succ_row[ib * stride].x;
                } else {
                    xin = succ_row[ib * stride];
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
                    const float2 cf = make_float2(edx[nc * 17 + tot_i], edy[nc * 17 + tot_i]);
                    add = cf.x * xin;
                    if (jd + 1 < d_wb) {
                        float xr;
                        if constexpr (HB) {
                            xr = succ_row[(ib + d_st) * stride].x;
                        } else {
                            xr = succ_row[(ib + d_st) * stride];
                        }
                        add = fmaf(cf.y, xr, add);
                    }
                }
                if constexpr (HB) {
                    v.x += add;
                } else {
                    v += add;
                }
            }
            out_row[j * stride] = v;
            // advance the multi-index over the emission box
#pragma unroll
            for (int c = C - 1; c >= 0; c--) {
                jc[c]++;
                ib += stb[c];
                if (jc[c] < bget(nx.w, c)) break;
                ib -= stb[c] * bget(nx.w, c);
                jc[c] = 0;
            }
        }
    }
}

// A read's emission factors as the engine reads them: the (mant, expo)
// table, and where present the window-normalised FP32 factors with their
// per-box exponent corrections (wp_window_factors_kernel).
struct ReadEmit {
    const EmitEntry* tab;  // [(t C + c) W + n]
    const float* gt;       // same layout, null when absent
    const uint8_t* gd;     // [(t C + c) W + u - 1]
    int W;
};

// Emission factors of the box nx at timestep t (at most 4 wide per channel,
// no interactions), per channel normalised by the box's largest exponent:
// g[c][k] for count L_c + k (0 beyond the box), and *kmax_out the sum of
// the normalising exponents.  gk is the (read, t)'s sum of window
// exponents: the window factors times 2^gdelta are these numbers exactly;
// with WP_GK_NONE they are normalised here from the table.  one: the
// (read, t)'s one-state factors (BatchArgs::gone).  Returns false
// when every factor of some channel is zero (only detected on the table
// path; on the other the zero factors give the pair P = 0 at this step's
// rescale).
template <int C>
__device__ __forceinline__ bool narrow_factors(const ReadEmit& re, int gk, float4 one, int t, PBox nx,
                                               float (&g)[C][4], int* kmax_out) {
    if constexpr (C <= 3) {
        // the read's box is one state in every channel: that state's factor
        // mantissas and exponent sum, as the two paths below would give
        if (__float_as_int(one.w) != WP_GK_NONE) {
            const float mv[3] = {one.x, one.y, one.z};
#pragma unroll
            for (int c = 0; c < C; c++) {
                g[c][0] = mv[c];
                g[c][1] = g[c][2] = g[c][3] = 0.0f;
            }
            *kmax_out = __float_as_int(one.w);
            return true;
        }
    }
    if (gk != WP_GK_NONE) {
        int kmax = gk;
#pragma unroll
        for (int c = 0; c < C; c++) {
            const int wc = bget(nx.w, c);
            const int base = (t * C + c) * re.W + bget(nx.lo, c);
            const int dl = re.gd[base + max(wc, 1) - 1];
            const float sc = exp2i(dl);
            const float* row = re.gt + base;
#pragma unroll
            for (int k = 0; k < 4; k++) g[c][k] = k < wc ? row[k] * sc : 0.0f;
            kmax -= dl;
        }
        *kmax_out = kmax;
        return true;
    }
    int kmax = 0;
#pragma unroll
    for (int c = 0; c < C; c++) {
        const EmitEntry* row = re.tab + (t * C + c) * re.W + bget(nx.lo, c);
        const int wc = bget(nx.w, c);
        EmitEntry en[4];
        int km = WP_EXPO_ZERO;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            en[k].mant = 0.0f;
            en[k].expo = WP_EXPO_ZERO;
            if (k < wc) en[k] = row[k];
            if (en[k].mant != 0.0f) km = max(km, en[k].expo);
        }
        if (km == WP_EXPO_ZERO) return false;
#pragma unroll
        for (int k = 0; k < 4; k++)
            g[c][k] = en[k].mant != 0.0f ? en[k].mant * exp2i(max(en[k].expo - km, -200)) : 0.0f;
        kmax += km;
    }
    *kmax_out = kmax;
    return true;
}

// Emission multiply for boxes at most 4 wide per channel without
// interactions (peptide-emission.cc:212-243): per channel the box's entries
// normalised by their largest exponent, in registers; the factor of state n
// is prod_c g[c][n_c - L_t] * 2^kmax, times sf (the pending rescale and
// folded coefficients).  Returns the sum of the multiplied states;
// *kmax_out receives the normalising exponent (WP_EXPO_ZERO: every factor
// of some channel is zero), *em0_out the all-zero state's factor when
// allow_t.  Out of line, as edman_gather.
template <int C, class V>
__device__ __noinline__ float emission_narrow(V* cur, int stride, int t, PBox nx, ReadEmit re, int gk, float4 one,
                                              bool allow_t, float sf, int* kmax_out, float* em0_out) {
    int kmax = 0;
    float part = 0.0f;
    float em0 = 0.0f;
    // Per channel: the box's entries normalised by their largest
    // exponent, in registers; the factor of state n is
    // prod_c g[c][n_c - L_t] * 2^kmax.
    float g[C][4];
    if (!narrow_factors<C>(re, gk, one, t, nx, g, &kmax)) {
        *kmax_out = WP_EXPO_ZERO;
        return 0.0f;
    }
    if (allow_t) {
        em0 = 1.0f;
#pragma unroll
        for (int c = 0; c < C; c++) em0 *= g[c][0];
    }
    // the pending rescale 2^-k_prev (1 - p) of the last timestep
    const int vn = bvol<C>(nx.w);
    int jc[C];
#pragma unroll
    for (int c = 0; c < C; c++) jc[c] = 0;
    for (int j = 0; j < vn; j++) {
        float w = sf;
#pragma unroll
        for (int c = 0; c < C; c++) {
            const int k = jc[c];
            w *= k == 0 ? g[c][0] : k == 1 ? g[c][1] : k == 2 ? g[c][2] : g[c][3];
        }
        V* col = cur + j * stride;
        for (int e = 0; e <= t; e++) {
            V s = vmul(w, col[e * vn * stride]);
            col[e * vn * stride] = s;
            part += vtotal(s);
        }
#pragma unroll
        for (int c = C - 1; c >= 0; c--) {
            if (++jc[c] < bget(nx.w, c)) break;
            jc[c] = 0;
        }
    }
    *kmax_out = kmax;
    *em0_out = em0;
    return part;
}

// Edman (edman-transition.cc:62-162) and emission (peptide-emission.cc:
// 212-243) of one timestep in one pass, for emission boxes at most 4 wide
// per channel without interactions: edman_gather followed by
// emission_narrow, with the emission box's state j outer and the Edman
// slice e inner, so that a state's index work (its place in the bleached
// box bx, its dye counts, the channels with a state one dye up) is done once
// per state instead of once per (state, slice), and the Edman output is
// multiplied by its emission factor before it is stored.  cur holds the
// bleached box (t >= 1 slices), nxt receives the emission box (t + 1
// slices).  codes: the pair's Edman code per position (PeptideRec::ecode),
// one byte per position at codes[k * stride]; a byte permute of the state's
// packed dye counts with the code byte as the selector gives the cut
// channel's count (and whether the state one dye up exists), so a slice
// costs no shifts of the packed dye sequence.  The bleached box's per-slice volume must be at
// most 255.  Returns the sum of the new states; *kmax_out the normalising
// exponent (WP_EXPO_ZERO: every factor of some channel is zero), *em0_out
// the all-zero state's factor.
template <int C, bool HB>
__device__ __forceinline__ float edman_emit(const typename StateOf<HB>::V* __restrict__ cur,
                                         typename StateOf<HB>::V* __restrict__ nxt, int stride, int t, PBox bx,
                                         PBox nx, const uint8_t* __restrict__ codes, const float* __restrict__ edx,
                                         const float* __restrict__ edy, float pf, const ReadEmit& re, int gk, float4 one, bool allow_t, float sf,
                                         int* kmax_out, float* em0_out) {
    using V = typename StateOf<HB>::V;
    // per channel: the box's emission entries normalised by their largest
    // exponent (as emission_narrow)
    float g[C][4];
    int kmax = 0;
    if (!narrow_factors<C>(re, gk, one, t, nx, g, &kmax)) {
        *kmax_out = WP_EXPO_ZERO;
        return 0.0f;
    }
    *kmax_out = kmax;
    if (allow_t) {
        float em0 = 1.0f;
#pragma unroll
        for (int c = 0; c < C; c++) em0 *= g[c][0];
        *em0_out = em0;
    }
    // the bleached box's strides, one byte per channel
    uint32_t stpk = 0;
    int vb = 1;
#pragma unroll
    for (int c = C - 1; c >= 0; c--) {
        stpk = bset(stpk, c, vb);
        vb *= bget(bx.w, c);
    }
    // the box's first state: bit 7 of byte c set where the bleached box is
    // wider than one in channel c (bytes of bx.w are at most 16, and 0 past
    // the channels, so no byte carries into the next)
    const uint32_t up0 = (bx.w + 0x7e7e7e7eu) & 0x80808080u;
    const int vn = bvol<C>(nx.w);
    const int sb = vb * stride, sn = vn * stride;
    float part = 0.0f;
    // The box's states in row-major order, as an odometer over the
    // channels: the state's index in the bleached box (ib), its packed
    // counts with the one-dye-up bits (X), and each channel's emission
    // factor (gc[c] = g[c][k_c]) are updated as the odometer turns; the
    // state's weight is sf g[0][k_0] ... g[C-1][k_{C-1}], multiplied in
    // that order.
    int jc[C];
    float gc[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
        jc[c] = 0;
        gc[c] = g[c][0];
    }
    int ib = 0;
    uint32_t X = nx.lo | up0;
    for (int j = 0; j < vn; j++) {
        float w = sf;
#pragma unroll
        for (int c = 0; c < C; c++) w *= gc[c];
        const V* cs = cur + ib * stride;  // slice e - 1 of the state's column
        V* out = nxt + j * stride;
        // Edman success into slice e from slice e - 1 (value prev, column
        // sp): the state's own count (x) and the state one dye up losing the
        // cut dye (y)
        auto success = [&](const uint8_t* cp, const V prev, const V* sp) -> float {
            const uint32_t code = *cp;
            // byte 0: the cut channel's count and its one-up bit (the code
            // byte is the selector; the other bytes are not used)
            const uint32_t b = prmt(X, 0u, code);
            const int ci = (int)(b & 0x7fu) * 17 + (int)(code >> 4);  // (count, tot)
            float xin;
            if constexpr (HB) {
                xin = prev.x;
            } else {
                xin = prev;
            }
            float add = edx[ci] * xin;
            if (b & 0x80u) {
                const V xr = sp[(int)(prmt(stpk, 0u, code) & 0xffu) * stride];
                if constexpr (HB) {
                    add = fmaf(edy[ci], xr.x, add);
                } else {
                    add = fmaf(edy[ci], xr, add);
                }
            }
            return add;
        };
        // slice 0: failure only
        V prev = cs[0];
        {
            V v;
            if constexpr (HB) {
                v = make_float2(pf * prev.x, prev.y);  // broken-N copied unchanged
            } else {
                v = pf * prev;
            }
            const V sv = vmul(w, v);
            out[0] = sv;
            part += vtotal(sv);
        }
        const uint8_t* cp = codes;
        // slices in pairs: two independent chains per step (and two sums)
        float part2 = 0.0f;
        int e = 1;
        for (; e + 1 < t; e += 2) {
            const V f0 = cs[sb], f1 = cs[2 * sb];
            const float a0 = success(cp, prev, cs);
            const float a1 = success(cp + stride, f0, cs + sb);
            V v0, v1;
            if constexpr (HB) {
                v0 = make_float2(fmaf(pf, f0.x, a0), f0.y);
                v1 = make_float2(fmaf(pf, f1.x, a1), f1.y);
            } else {
                v0 = fmaf(pf, f0, a0);
                v1 = fmaf(pf, f1, a1);
            }
            const V s0 = vmul(w, v0), s1 = vmul(w, v1);
            out[e * sn] = s0;
            out[(e + 1) * sn] = s1;
            part += vtotal(s0);
            part2 += vtotal(s1);
            prev = f1;
            cs += 2 * sb;
            cp += 2 * stride;
        }
        if (e < t) {
            const float add = success(cp, prev, cs);
            cs += sb;
            cp += stride;
            const V f = *cs;
            V v;
            if constexpr (HB) {
                v = make_float2(fmaf(pf, f.x, add), f.y);
            } else {
                v = fmaf(pf, f, add);
            }
            prev = f;
            const V sv = vmul(w, v);
            out[e * sn] = sv;
            part += vtotal(sv);
        }
        part += part2;
        {
            // slice t: success only (the bleached box has t slices)
            const float add = success(cp, prev, cs);
            V v;
            if constexpr (HB) {
                v = make_float2(add, 0.0f);
            } else {
                v = add;
            }
            const V sv = vmul(w, v);
            out[t * sn] = sv;
            part += vtotal(sv);
        }
        if (j + 1 < vn) {
            bool carry = true;
#pragma unroll
            for (int c = C - 1; c >= 0; c--) {
                if (carry) {
                    const int st_c = bget(stpk, c);
                    const int k = jc[c] + 1;
                    if (k < bget(nx.w, c)) {
                        jc[c] = k;
                        ib += st_c;
                        X += 1u << (8 * c);
                        if (k + 1 >= bget(bx.w, c)) X &= ~(0x80u << (8 * c));
                        gc[c] = k == 1 ? g[c][1] : k == 2 ? g[c][2] : g[c][3];
                        carry = false;
                    } else {
                        // channel c back to its first count (its one-up bit
                        // as for the box's first state)
                        ib -= jc[c] * st_c;
                        X = (X - ((uint32_t)jc[c] << (8 * c))) | (up0 & (0x80u << (8 * c)));
                        jc[c] = 0;
                        gc[c] = g[c][0];
                    }
                }
            }
        }
    }
    return part;
}

// Runs one pair.  Returns 1 when its boxes exceed the slab (nothing
// written), else 0 with P = *mant * 2^*expo (mant == 0: P == 0).
template <int C, bool HB>
__device__ int engine_pair(const BatchArgs& a, const SmemModel& M, int r,
                           const PeptideRec& pep, typename StateOf<HB>::V* slab, uint8_t* codes, int stride,
                           int half, int vmax, float* out_mant, int* out_expo) {
    using V = typename StateOf<HB>::V;
    const DevModel& m = *a.model;
    // model scalars in registers (stores to the slab cannot move them)
    const int T = m.T;
    const float pf = m.pf;
    const bool interacting = m.interacting != 0;
    const EmitEntry* tab = a.tab + (long)r * a.entries;
    ReadEmit re;
    re.tab = tab;
    re.W = a.W;
    re.gt = a.gtab ? a.gtab + (long)r * a.entries : nullptr;
    re.gd = a.gdelta ? a.gdelta + (long)r * a.entries : nullptr;
    const int* gKr = a.gtab ? a.gK + (long)r * T : nullptr;
    const float4* gOr = a.gone ? a.gone + (long)r * T : nullptr;
    const uint32_t* Lpk = a.Lpk + (long)r * T;
    const uint32_t* Upk = a.Upk + (long)r * T;
    uint32_t D1 = 0;  // D_c + 1 per channel, packed
#pragma unroll
    for (int c = 0; c < C; c++) D1 = bset(D1, c, pep.D[c] + 1);
    // Emission box of timestep t: [L_t, min(U_t, D + 1)), packed.
    // All bytes are below 128 (counts and bounds are at most 16, 0 past the
    // channels), so byte-wise min and difference work on the whole word: bit
    // 7 of (uw | 0x80...) - D1 is set in byte c exactly where U >= D + 1, no
    // borrow crosses a byte, and min(U, D + 1) > L for a live pair.
    auto box_of = [&](uint32_t lw, uint32_t uw) {
        PBox b;
        b.lo = lw & 0x7f7f7f7fu;  // bit 31 of the word is the allow flag
        const uint32_t msk = ((((uw | 0x80808080u) - D1) >> 7) & 0x01010101u) * 0xffu;
        b.w = ((D1 & msk) | (uw & ~msk)) - b.lo;
        return b;
    };
    auto emission_box = [&](int t) { return box_of(Lpk[t], Upk[t]); };

    // The largest box any step of this pair uses (pair_vmax, left with the
    // pair by the compaction: item_slot) must fit the slab half; a pair
    // that does not is handed to the next pass before anything is written.
    if (vmax > half) return 1;
    // Dye channel and remaining dyes of that channel per Edman position,
    // packed 4 bits each (positions < 16) so the Edman loop reads registers.
    const bool pk = T <= 17;
    const uint64_t dye_pk = pep.dye_pk, tot_pk = pep.tot_pk;
    if (pk) {
        // the Edman code of each position, one byte per position in the
        // thread's slice of shared memory (read by edman_emit)
        const uint64_t ec0 = pep.ecode[0], ec1 = pep.ecode[1];
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (k < T - 1) codes[k * stride] = (uint8_t)((k < 8 ? ec0 : ec1) >> (8 * (k & 7)));
    }

    V* cur = slab;
    V* nxt = slab + half * stride;

    // ---- t = 0: the start state (0, D) (peptide-state-vector.cc:38-40),
    // the initial block (block-transition.cc:33-62) and the dud steps
    // (dud-transition.cc:25-37).  From a single state the duds give state n
    // of the emission box [L_0, min(U_0, D + 1)) the start value times
    // prob(D_c -> n_c) of each channel in turn: the reference's
    // channel-by-channel passes multiply the same factors in the same order,
    // and states outside the box are pruned, so the box is written directly.
    PBox bx = emission_box(0);
    {
        const int v = bvol<C>(bx.w);
        int jc[C];
#pragma unroll
        for (int c = 0; c < C; c++) jc[c] = 0;
        for (int j = 0; j < v; j++) {
            V s;
            if constexpr (HB) {
                s = make_float2(1.0f - m.p_ib, m.p_ib);
            } else {
                s = 1.0f;
            }
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int d = pep.D[c], n = bget(bx.lo, c) + jc[c];
                s = vmul(M.dud[c][d * (d + 1) / 2 + n], s);
            }
            cur[j * stride] = s;
#pragma unroll
            for (int c = C - 1; c >= 0; c--) {
                if (++jc[c] < bget(bx.w, c)) break;
                jc[c] = 0;
            }
        }
    }
    // A binomial step along a channel whose input and output boxes are both
    // one wide is one coefficient for the whole state: it is carried in
    // bscale and applied with the next emission multiply instead of a pass.
    float bscale = 1.0f;
    uint32_t fold_lo = 0xffffffffu;  // corner of the cached folded bleach product
    float fold_k = 1.0f;

    int expo = 0;           // the true state is the stored state times 2^expo
    float pd = 0.0f;        // detached state, in the rescaled frame
    int k_prev = 0;         // exponent removed at the last rescale
    float scale_prev = 1.0f;  // 2^-k_prev (exp2i clamps at 2^127 as the multiplier did)
    float fac_prev = 1.0f;  // (1 - p_detach) pending from the last timestep
    // Closes timestep t after its emission multiply: the detached state
    // (kept only while the box includes zero, peptide-emission.cc:218-223),
    // the exact power-of-two rescale and the next timestep's detach folded
    // into the rescaled frame (detach-transition.cc:36-68).  Returns true
    // when the pair is finished (result written).
    auto close_step = [&](int t, float part, float em0, int kmax, bool allow_t) -> bool {
        pd = allow_t ? pd * em0 : 0.0f;
        expo += kmax;
        const float tot = part + pd;
        if (!(tot > 0.0f) || !isfinite(tot)) {
            *out_mant = 0.0f;
            *out_expo = 0;
            return true;
        }
        // tot = fm * 2^k, fm in [0.5, 1) (frexpf; normal numbers from the bits)
        int k;
        float fm;
        const int bits = __float_as_int(tot);
        if (bits >= 0x00800000) {
            k = (bits >> 23) - 126;
            fm = __int_as_float((bits & 0x007fffff) | 0x3f000000);
        } else {
            fm = frexpf(tot, &k);
        }
        if (t == T - 1) {
            *out_mant = fm;
            *out_expo = expo + k;
            return true;
        }
        expo += k;
        const float f = exp2i(-k);
        // p_detached += p * sum of the states
        pd = (pd + M.p_det[t] * part) * f;
        k_prev = k;
        scale_prev = f;
        fac_prev = 1.0f - M.p_det[t];
        return false;
    };
    uint32_t lw_next = Lpk[0], uw_next = Upk[0];
    int gk_next = gKr ? gKr[0] : WP_GK_NONE;
    const float4 one_none = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(WP_GK_NONE));
    float4 one_next = gOr ? gOr[0] : one_none;
    int t = 0;
    for (;;) {
        // this timestep's box words; the next timestep's are fetched now so
        // their latency hides behind this timestep's work
        const uint32_t lw = lw_next, uw = uw_next;
        const int gk = gk_next;
        const float4 one = one_next;
        if (t + 1 < T) {
            lw_next = Lpk[t + 1];
            uw_next = Upk[t + 1];
            if (gKr) gk_next = gKr[t + 1];
            if (gOr) one_next = gOr[t + 1];
        }
        const PBox nx = box_of(lw, uw);
        const bool allow_t = (lw >> 31) != 0;
        // every channel of the emission box at most 4 wide (bytes below 128:
        // byte + 123 reaches bit 7 exactly from 5 up, no carry)
        const bool narrow = !interacting && ((nx.w + 0x7b7b7b7bu) & 0x80808080u) == 0;
        int kmax = 0;
        float part = 0.0f;
        float em0 = 0.0f;
        bool fused = false;  // Edman and emission done together (edman_emit)
        if (t > 0) {
            bscale = 1.0f;
            // Cyclic block (block-transition.cc:33-62) over e < t and the
            // previous emission box.
            if constexpr (HB) {
                if (m.p_cb != 0.0f) {
                    const int n = t * bvol<C>(bx.w);
                    for (int i = 0; i < n; i++) {
                        float2 s = cur[i * stride];
                        cur[i * stride] = make_float2((1.0f - m.p_cb) * s.x, s.y + m.p_cb * s.x);
                    }
                }
            }
            // Detach (detach-transition.cc:36-68) was folded into the last
            // rescale: pd already holds it, fac_prev carries (1 - p).
            // Bleach per channel: channel c moves from the previous box to
            // [L_t, min(U_t + 1, U_{t-1})).  L_t <= L_{t-1} (a suffix
            // maximum), so a channel one wide in the previous box stays one
            // wide exactly when L_t = L_{t-1}; when that holds for every
            // channel (most timesteps) the step is one coefficient per
            // channel, prob(L -> L), and the box does not change.
            if ((bx.w & chan_mask<C>()) == (0x01010101u & chan_mask<C>()) &&
                ((bx.lo ^ nx.lo) & chan_mask<C>()) == 0) {
                // the product over channels depends on L_t alone: kept from
                // the last timestep that folded the same corner
                if (nx.lo != fold_lo) {
                    fold_lo = nx.lo;
                    fold_k = 1.0f;
#pragma unroll
                    for (int c = 0; c < C; c++) {
                        const int l = bget(nx.lo, c);
                        fold_k *= M.bleach[c][l * (l + 3) / 2];
                    }
                }
                bscale = fold_k;
            } else
#pragma unroll 1
            for (int c = 0; c < C; c++) {
                const int ln = bget(nx.lo, c);
                const int bu = min(ln + bget(nx.w, c) + 1, bget(bx.lo, c) + bget(bx.w, c));
                if (bget(bx.w, c) == 1 && bu - ln == 1) {
                    const int from = bget(bx.lo, c);
                    bscale *= from >= ln ? M.bleach[c][from * (from + 1) / 2 + ln] : 0.0f;
                } else {
                    binomial_step<C, V>(cur, nxt, stride, t, bx, c, ln, bu - ln, M.bleach[c]);
                    V* tmp = cur;
                    cur = nxt;
                    nxt = tmp;
                }
                bx.lo = bset(bx.lo, c, ln);
                bx.w = bset(bx.w, c, bu - ln);
            }
            // Edman (edman-transition.cc:62-162) as a gather from slices e-1
            // (success) and e (failure) of the bleached box into the
            // emission box; both boxes share the lower corner L_t.
            // (with C <= 3 the bleached box of a narrow emission box is at
            // most 5^3 states per slice)
            fused = pk && narrow && (C <= 3 || bvol<C>(bx.w) <= 255);
            if (fused) {
                part = edman_emit<C, HB>(cur, nxt, stride, t, bx, nx, codes, M.edx, M.edy, pf, re, gk, one,
                                         allow_t, fac_prev * bscale * scale_prev, &kmax, &em0);
                if (kmax == WP_EXPO_ZERO) {
                    *out_mant = 0.0f;
                    *out_expo = 0;
                    return 0;
                }
            } else {
                edman_gather<C, HB>(cur, nxt, stride, t, bx, nx, pk, dye_pk, tot_pk, pep, M.edx, M.edy, pf);
            }
            V* tmp = cur;
            cur = nxt;
            nxt = tmp;
            bx = nx;
        }
        // ---- Emission t (peptide-emission.cc:212-243).  Factors normalised
        // by the largest exponent over the pair's box (a power of two, carried
        // in expo); the pending rescale is folded into the multiplier.
        if (fused) {
            // edman_emit applied the emission
        } else if (narrow) {
            part = emission_narrow<C, V>(cur, stride, t, nx, re, gk, one, allow_t,
                                         fac_prev * bscale * scale_prev, &kmax, &em0);
            if (kmax == WP_EXPO_ZERO) {
                *out_mant = 0.0f;
                *out_expo = 0;
                return 0;
            }
        } else {
            part = emission_table<C, V>(cur, stride, t, nx, a.W, tab, interacting, fac_prev * bscale, k_prev,
                                        &kmax, &em0);
            if (kmax == WP_EXPO_ZERO) {
                *out_mant = 0.0f;
                *out_expo = 0;
                return 0;
            }
            if (!allow_t) em0 = 0.0f;
        }
        if (close_step(t, part, em0, kmax, allow_t)) return 0;
        ++t;
    }
}

// Lists one engine pass reads and spills to.
struct EngineLists {
    const int2* in;
    const int* in_count;
    int* in_head;
    int2* out;
    int* out_count;
    int slab_half;
    int scr_floats;   // reserved per-thread scratch (floats), 0 when unused
    int spill_error;  // nonzero: nothing downstream takes spills; flag err
};

// Persistent: each warp takes 32 consecutive work items at a time.
template <int C, bool HB>
__global__ void __launch_bounds__(WP_ENGINE_THREADS) wp_engine_kernel(BatchArgs a, EngineLists L) {
    using V = typename StateOf<HB>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemModel& M = *reinterpret_cast<SmemModel*>(smem_raw);
    load_smem_model(M, *a.model);
    __syncthreads();
    const int nt = blockDim.x;
    V* slab_region = reinterpret_cast<V*>(smem_raw + ((sizeof(SmemModel) + 15) & ~(size_t)15));
    V* slab = slab_region + threadIdx.x;
    // per-thread Edman code bytes after the slabs (wp_engine_smem_bytes)
    uint8_t* codes = reinterpret_cast<uint8_t*>(slab_region + 2 * (size_t)L.slab_half * nt) + threadIdx.x;
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
            int vmax;
            const int p = slot_pep(a, rg.x, item_slot(a, rg, &vmax));
            float mant;
            int ex;
            int ov = engine_pair<C, HB>(a, M, rg.x, a.peps[p], slab, codes, nt, L.slab_half, vmax, &mant, &ex);
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

// Shared memory of one engine CTA: the model, two slab halves per thread,
// 16 Edman code bytes per thread and scr_floats more words per thread.
size_t wp_engine_smem_bytes(int slab_half, int scr_floats, bool has_block, int threads) {
    size_t elem = has_block ? sizeof(float2) : sizeof(float);
    return ((sizeof(SmemModel) + 15) & ~(size_t)15) + (size_t)2 * slab_half * threads * elem +
           (size_t)WP_ENGINE_CODES * threads + (size_t)scr_floats * threads * sizeof(float);
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
