// wp_common.cuh -- device-side data layout shared by the HMM kernels.
//
// Layout in HBM (all arrays are flat, one record per read / peptide):
//   DevModel        one per context: binomial dud/bleach tables per channel
//                   (triangular, UniversalPrecomputations), detach rate per
//                   timestep (DecayingRateModel), Edman failure, block rates.
//   PeptideRec      one per dye-seq: dye count per channel, dye channel at
//                   each Edman position < T and the remaining dyes of that
//                   channel there (DyeTrack(e, c) for c = dye_seq[e]).
//   ReadRec         one per radiometry, written by the prep kernel: the
//                   emission box [cmin, cmax) per (t, c) and the emission
//                   factors as (mantissa, exponent) pairs -- per (t, c, n)
//                   when the channels do not interact, else per (t, n-vector).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/whatprot_gb300.h"
#include "wp_kdtree.h"

#define WP_W (WP_MAX_DYES_PER_CHANNEL + 1)      // extent cap per channel
#define WP_TRI (WP_W * (WP_W + 1) / 2)          // triangular table size
#define WP_MAX_TIERS 5                          // engine passes the compaction routes to
// Batch counters: [2k, 2k + 1] list count / head of engine pass k, then the
// dense kernel's count / head, then the non-empty pairs.
#define WP_CNT_DENSE (2 * WP_MAX_TIERS)
#define WP_CNT_LIVE (2 * WP_MAX_TIERS + 2)
#define WP_CNT_N (2 * WP_MAX_TIERS + 3)
#define WP_GROUP_WARPS 8      // warps per CTA of wp_compact_groups_kernel (one read at a time each)
#define WP_GROUP_MAX 512      // dye-count vectors (groups) that kernel takes
#define WP_GROUP_PERM_SMEM 8192  // peptides up to which it stages the shape order in shared memory

struct DevModel {
    int C;
    int T;
    int has_block;        // p_initial_block != 0 || p_cyclic_block != 0
    int interacting;      // any interaction factor != 1
    float pf;             // p_edman_failure
    float p_ib;           // p_initial_block
    float p_cb;           // p_cyclic_block
    float p_det[WP_MAX_TIMESTEPS];      // p_detach[t]
    float dud[WP_MAX_CHANNELS][WP_TRI];    // prob(from, to) at from*(from+1)/2+to
    float bleach[WP_MAX_CHANNELS][WP_TRI];
    // Emission model (FP64: the emission factors are computed as the
    // reference does, then rounded once).
    double bg_sig[WP_MAX_CHANNELS];
    double sig[WP_MAX_CHANNELS];
    double mu[WP_MAX_CHANNELS];
    double inter[WP_MAX_CHANNELS][WP_MAX_CHANNELS];
    double flat[WP_MAX_CHANNELS][WP_MAX_CHANNELS];
    // Without interactions ChannelModel's per-count quantities depend on the
    // channel and the count n alone (channel-model.h:35-70), so they are
    // tabulated once per model for n = 0 .. WP_W: adjusted mu, sigma,
    // 1 / (sigma sqrt(2 pi)) and 2 sigma^2 (wp_fill_emission_tables).
    double e_amu[WP_MAX_CHANNELS][WP_W + 1];
    double e_sig[WP_MAX_CHANNELS][WP_W + 1];
    double e_norm[WP_MAX_CHANNELS][WP_W + 1];
    double e_den[WP_MAX_CHANNELS][WP_W + 1];
    double e_l2den[WP_MAX_CHANNELS][WP_W + 1];  // log2(e) / e_den: the pdf's exponent in base 2
};

// Host side: fills the e_* tables of a non-interacting model from mu, sig
// and bg_sig with the operations and order of ChannelModel::adjusted_mu,
// sigma and pdf_helper.
inline void wp_fill_emission_tables(DevModel& m) {
    const double pi = 3.141592653589793238;
    for (int c = 0; c < m.C; c++)
        for (int n = 0; n <= WP_W; n++) {
            const double amu = m.mu[c] * (double)n;
            const double bg2 = m.bg_sig[c] * m.bg_sig[c];
            const double var = amu * m.sig[c] * m.sig[c];
            const double s = sqrt(bg2 + var);
            m.e_amu[c][n] = amu;
            m.e_sig[c][n] = s;
            m.e_norm[c][n] = 1.0 / (s * sqrt(2.0 * pi));
            m.e_den[c][n] = 2.0 * s * s;
            m.e_l2den[c][n] = 1.4426950408889634074 / m.e_den[c][n];
        }
}

// BinomialTransition::reserve (hmm/step/binomial-transition.cc:51-67): the
// triangular table prob(from, to) of `to` of `from` dyes surviving (each
// lost with probability q), from an FP64 running row updated in place and
// rounded once into the FP32 output (no allocation).
inline void wp_binomial_table(double q, int max_n, float* out) {
    double row[WP_MAX_DYES_PER_CHANNEL + 1];
    const double p = 1.0 - q;
    row[0] = 1.0;
    out[0] = 1.0f;
    for (int i = 1; i <= max_n; i++) {
        const double prev_diag = row[i - 1];
        for (int j = i - 1; j >= 1; j--) row[j] = row[j] * q + row[j - 1] * p;
        row[0] = row[0] * q;
        row[i] = prev_diag * p;
        for (int j = 0; j <= i; j++) out[i * (i + 1) / 2 + j] = (float)row[j];
    }
}

// The device model of a SequencingModel for T timesteps (the model part of
// UniversalPrecomputations, hmm/precomputations/universal-precomputations.cc:
// 23-59): FP32 rates, detach rate per timestep (DecayingRateModel,
// decaying-rate-model.cc:47-50), binomial dud/bleach tables, the FP64
// emission model and its per-count tables.  Host only; allocates nothing.
// Returns WP_OK, or the status for a shape or a null array it does not take.
inline wp_status wp_fill_dev_model(const wp_seq_model* m, int T, DevModel* hp) {
    const int C = m->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS || T < 1 || T > WP_MAX_TIMESTEPS) return WP_ERR_UNSUPPORTED;
    if (!m->p_bleach || !m->p_dud || !m->bg_sig || !m->mu || !m->sig) return WP_ERR_INVALID;
    DevModel& h = *hp;
    memset(&h, 0, sizeof(h));
    h.C = C;
    h.T = T;
    h.pf = (float)m->p_edman_failure;
    h.p_ib = (float)m->p_initial_block;
    h.p_cb = (float)m->p_cyclic_block;
    h.has_block = (m->p_initial_block != 0.0 || m->p_cyclic_block != 0.0) ? 1 : 0;
    for (int t = 0; t < T; t++)
        h.p_det[t] = (float)(m->p_detach + m->p_initial_detach * exp(-(double)t * m->p_initial_detach_decay));
    h.interacting = 0;
    for (int c = 0; c < C; c++) {
        wp_binomial_table(m->p_dud[c], WP_MAX_DYES_PER_CHANNEL, h.dud[c]);
        wp_binomial_table(m->p_bleach[c], WP_MAX_DYES_PER_CHANNEL, h.bleach[c]);
        h.bg_sig[c] = m->bg_sig[c];
        h.sig[c] = m->sig[c];
        h.mu[c] = m->mu[c];
        for (int o = 0; o < C; o++) {
            h.inter[c][o] = m->interactions ? m->interactions[c * C + o] : 1.0;
            h.flat[c][o] = m->flat_interactions ? m->flat_interactions[c * C + o] : 1.0;
            if (h.inter[c][o] != 1.0 || h.flat[c][o] != 1.0) h.interacting = 1;
        }
    }
    wp_fill_emission_tables(h);
    return WP_OK;
}

// One peptide.  dye[e] is the channel removed by a successful Edman cycle at
// position e (-1 none), tot[e] = DyeTrack(e, dye[e]).
struct PeptideRec {
    uint8_t D[WP_MAX_CHANNELS];
    int8_t dye[WP_MAX_TIMESTEPS];
    uint8_t tot[WP_MAX_TIMESTEPS];
    // Positions 0..15 packed 4 bits each (the engine reads these when
    // T <= 17): dye_pk nibble e = dye[e] + 1, tot_pk nibble e = tot[e].
    uint64_t dye_pk;
    uint64_t tot_pk;
    // The same positions as one Edman code byte each (ecode[0]: positions
    // 0..7, ecode[1]: 8..15): (tot << 4) | channel for a dye, 4 for none.
    // The engine's Edman step reads the coefficient row tot and, through a
    // byte permute with the code byte itself as the selector, the dye count
    // of the cut channel in the result's byte 0 (selector nibble 0 is the
    // channel, its sign-extension bit clear; for none it is 4, the constant
    // zero byte; the result's other bytes are not used).
    uint64_t ecode[2];
};

// Fills dye_pk / tot_pk / ecode from dye[] and tot[] (tot <= 15 per channel).
__host__ __device__ inline void wp_pack_peptide(PeptideRec& r) {
    uint64_t d = 0, t = 0;
    uint64_t ec[2] = {0, 0};
    for (int e = 0; e < 16 && e < WP_MAX_TIMESTEPS; e++) {
        d |= (uint64_t)((r.dye[e] + 1) & 15) << (4 * e);
        t |= (uint64_t)(r.tot[e] & 15) << (4 * e);
        const uint64_t code = r.dye[e] >= 0 ? (uint64_t)(((r.tot[e] & 15) << 4) | (r.dye[e] & 3)) : 4u;
        ec[e >> 3] |= code << (8 * (e & 7));
    }
    r.dye_pk = d;
    r.tot_pk = t;
    r.ecode[0] = ec[0];
    r.ecode[1] = ec[1];
}

// Emission factor of one table entry: value = mant * 2^expo exactly as the
// reference's FP64 product, mant in [0.5, 1) rounded to FP32; mant == 0 means
// the entry is zero (outside the pruning box, or underflowed in FP64).
struct EmitEntry {
    float mant;
    int expo;
};

#define WP_EXPO_ZERO (-100000)
#define WP_GK_NONE (-2147483647 - 1)  // gK: no window factors for this (read, t)

__host__ __device__ inline int wp_ipow(int b, int e) {
    int r = 1;
    for (int i = 0; i < e; i++) r *= b;
    return r;
}

// Size of one read's slab of emission entries.
__host__ __device__ inline int wp_read_table_entries(int T, int C, int W, int interacting) {
    return interacting ? T * wp_ipow(W, C) : T * C * W;
}

// Model tables a CTA keeps in shared memory.
struct SmemModel {
    float dud[WP_MAX_CHANNELS][WP_TRI];
    float bleach[WP_MAX_CHANNELS][WP_TRI];
    float p_det[WP_MAX_TIMESTEPS];
    // Edman success coefficients (edman-transition.cc:62-162) at
    // [n * 17 + tot]: for a state with n dyes left of the channel cut at a
    // position with tot dyes of that channel remaining, edx = (1 - p_fail) *
    // (tot - n) / tot (the cut dye was another one) and edy = (1 - p_fail) *
    // (n + 1) / tot (the state one dye up lost the cut dye).  tot = 0 (no dye
    // at the position): edx = 1 - p_fail, edy = 0.  Rows of 17 words: the
    // lanes of a warp (pairs of one read, different peptides) mostly read
    // one count n at different tot, which then fall in different banks.
    float edx[16 * 17];
    float edy[16 * 17];
};

// Everything one batch of reads needs on the device.  Per-read arrays are
// indexed [r][t][c] (uint8) or [r][t]; per-slot arrays by the slot g: the
// slots of read r are [slot_off[r], slot_off[r+1]) (all-peptides mode:
// slot_off == null, slots r*P .. r*P+P-1 and slot g holds peptide g - r*P).
struct BatchArgs {
    const DevModel* model;
    const PeptideRec* peps;
    const int* counts;         // peptide multiplicities
    int R;
    int P;
    int W;                     // Dmax + 1
    int entries;               // emission entries per read
    const uint8_t* lo;         // cmin per (r, t, c)
    const uint8_t* hi;         // cmax
    uint8_t* Lsuf;             // max_{t' >= t} cmin
    uint8_t* Upre;             // min_{t' <= t} cmax
    uint8_t* allow;            // per (r, t): the emission box includes zero
    uint32_t* Lpk;             // per (r, t): L per channel in bits 8c..8c+6, bit 31 = allow
    uint32_t* Upk;             // per (r, t): U byte per channel
    uint8_t* flags;            // per r: bit 0 = the read prunes every pair
    const EmitEntry* tab;      // per read: emission factors
    // Non-interacting models (all null otherwise, or where unused): per
    // (r, t, c, n) the emission factor normalised over the read's pruning
    // window [cmin, cmax) of (t, c), in FP32 (gtab); per (r, t) the sum over
    // channels of the windows' normalising exponents (gK), or WP_GK_NONE
    // when some factor lies more than 2^100 below its window's largest; per
    // (r, t, c) and box [L_t, u), u in (L_t, U_t], the window's exponent
    // minus the box's at byte u - 1 (gdelta).  Written by
    // wp_window_factors_kernel; the engine scales them instead of
    // normalising each pair's box itself.
    float* gtab;
    uint8_t* gdelta;
    int* gK;
    // per (r, t), with gtab, C <= 3: where the read's box [L_t, U_t) is one
    // state in every channel (so is every non-empty pair's), that state's
    // factor mantissa per channel (x, y, z) and the sum of its exponents in
    // w (int bits); w = WP_GK_NONE otherwise
    float4* gone;
    const int* cand;           // per slot: peptide index (null: all peptides)
    const int* perm;           // all-peptides mode: peptides in shape order (or null)
    const int* shape_rank;     // candidate mode: each peptide's position in that order (or null)
    const uint32_t* uniq_D;    // distinct dye-count vectors, byte c = channel c (or null)
    const int* pep_u;          // per peptide: its vector's index in uniq_D
    int n_uniq;
    // All-peptides mode: the runs of perm with one dye-count vector
    // ("groups"): group u is perm[grp_start[u] .. grp_start[u + 1]) with
    // vector grp_D[u] (byte c = channel c).
    const int* grp_start;
    const uint32_t* grp_D;
    int n_grp;
    // Result indices.  pair_info null: a pair's result index is its slot
    // g, work items are (r, g), every slot gets a result, and the pair's
    // largest box waits in res_expo[g] for the engine.  pair_info set
    // (wp_compact_groups_kernel): only non-empty pairs get a result index;
    // read r's are rd_base[r] .. rd_base[r] + rd_n[r] - 1, in the
    // compaction's order; work items are (r, d) and pair_info[d] = (the
    // pair's slot offset within its read, its largest box); a pair without
    // one has P = 0.
    int2* pair_info;
    int* rd_base;
    int* rd_n;
    // nonzero (wp_engine_replay, pair_info null): the engine passes run
    // lists whose pairs they have run before, so the result slot holds a
    // result, not the routed box size; the slot is still read, its value
    // ignored
    int replay_trust;
    const int* slot_off;       // [R + 1] or null
    float* res_mant;           // per result index: P = res_mant * 2^res_expo
    int* res_expo;
    int2* work;                // non-empty pairs (r, result index)
    int* work_count;
    int* work_head;
    int2* ovf;                 // pairs whose state exceeds the thread slab
    int* ovf_count;
    int* ovf_head;
    int* err;
    int slab_half;             // per-thread slab half, in state elements
    int dense_S_cap;           // overflow kernel: max states per Edman slice
    // Routing by the compaction over the engine passes ("tiers", in launch
    // order; n_tiers == 0: every live pair to `work`): a pair goes to the
    // list of the first tier whose slab half holds its largest box
    // (pair_vmax), else to `ovf` (the dense kernel; route_dense == 0: none,
    // the pair gets P = 0 and err = 2).
    int n_tiers;
    int tier_half[WP_MAX_TIERS];
    int2* tier_list[WP_MAX_TIERS];
    int* tier_count[WP_MAX_TIERS];
    int route_dense;
    int* live_count;           // non-empty pairs (nullable)
};

// Largest state box, in elements with the Edman slices counted, that any
// step of a pair uses: the emission box of t = 0 (the engine writes the
// start state after its duds directly there), and per timestep t >= 1
// the previous emission box, the bleach output / Edman input box
// [L_t, min(U_t + 1, U_{t-1})), the boxes in between (channels bleached so
// far at their new width, the others at the old) and the emission box,
// with U clamped to D + 1.  Lw / Uw are the read's packed box words.
__device__ inline int pair_vmax(int C, int T, const uint32_t* Lw, const uint32_t* Uw, const uint8_t* D) {
    int lo_p[WP_MAX_CHANNELS], w_p[WP_MAX_CHANNELS];
    int vmax = 1;
    for (int c = 0; c < C; c++) {
        const int d1 = D[c] + 1;
        const int l = (int)((Lw[0] >> (8 * c)) & 0x7fu);
        lo_p[c] = l;
        w_p[c] = min((int)((Uw[0] >> (8 * c)) & 0xffu), d1) - l;
        vmax *= w_p[c];
    }
    for (int t = 1; t < T; t++) {
        const uint32_t lw = Lw[t], uw = Uw[t];
        int vp = t, vb = t, vn = t + 1, vm = t;
        for (int c = 0; c < C; c++) {
            const int ln = (int)((lw >> (8 * c)) & 0x7fu);
            const int wn = min((int)((uw >> (8 * c)) & 0xffu), D[c] + 1) - ln;
            const int wb = min(ln + wn + 1, lo_p[c] + w_p[c]) - ln;
            vp *= w_p[c];
            vb *= wb;
            vn *= wn;
            vm *= max(wb, w_p[c]);
            lo_p[c] = ln;
            w_p[c] = wn;
        }
        vmax = max(vmax, max(max(vp, vb), max(vn, vm)));
    }
    return vmax;
}

// pair_vmax with the channel count fixed and the dye counts packed one per
// byte (register arithmetic only; pair_vmax_w picks C at run time).
template <int C>
__device__ __forceinline__ int pair_vmax_c(int T, const uint32_t* Lw, const uint32_t* Uw, uint32_t Dw) {
    int lo_p[C], w_p[C], d1[C];
    int vmax = 1;
#pragma unroll
    for (int c = 0; c < C; c++) {
        d1[c] = (int)((Dw >> (8 * c)) & 0xffu) + 1;
        const int l = (int)((Lw[0] >> (8 * c)) & 0x7fu);
        lo_p[c] = l;
        w_p[c] = min((int)((Uw[0] >> (8 * c)) & 0xffu), d1[c]) - l;
        vmax *= w_p[c];
    }
    for (int t = 1; t < T; t++) {
        const uint32_t lw = Lw[t], uw = Uw[t];
        int vp = t, vb = t, vn = t + 1, vm = t;
#pragma unroll
        for (int c = 0; c < C; c++) {
            const int ln = (int)((lw >> (8 * c)) & 0x7fu);
            const int wn = min((int)((uw >> (8 * c)) & 0xffu), d1[c]) - ln;
            const int wb = min(ln + wn + 1, lo_p[c] + w_p[c]) - ln;
            vp *= w_p[c];
            vb *= wb;
            vn *= wn;
            vm *= max(wb, w_p[c]);
            lo_p[c] = ln;
            w_p[c] = wn;
        }
        vmax = max(vmax, max(max(vp, vb), max(vn, vm)));
    }
    return vmax;
}

__device__ __forceinline__ int pair_vmax_w(int C, int T, const uint32_t* Lw, const uint32_t* Uw, uint32_t Dw) {
    switch (C) {
        case 1: return pair_vmax_c<1>(T, Lw, Uw, Dw);
        case 2: return pair_vmax_c<2>(T, Lw, Uw, Dw);
        case 3: return pair_vmax_c<3>(T, Lw, Uw, Dw);
        default: return pair_vmax_c<4>(T, Lw, Uw, Dw);
    }
}

__host__ __device__ inline int slot_begin(const BatchArgs& a, int r) {
    return a.slot_off ? a.slot_off[r] : r * a.P;
}
__host__ __device__ inline int slot_pep(const BatchArgs& a, int r, int g) {
    return a.cand ? a.cand[g] : g - r * a.P;
}
// The slot of work item rg = (r, result index) and the pair's largest box
// (BatchArgs::pair_info).
__device__ __forceinline__ int item_slot(const BatchArgs& a, int2 rg, int* vmax) {
    if (a.pair_info) {
        const int2 inf = a.pair_info[rg.y];
        *vmax = inf.y;
        return slot_begin(a, rg.x) + inf.x;
    }
    *vmax = a.res_expo[rg.y] & (a.replay_trust ? 0 : -1);
    return rg.y;
}

// 2^x as a float for x <= 127 (0 below the subnormal range).
__device__ __forceinline__ float exp2i(int x) {
    x = min(x, 127);
    if (x >= -126) return __int_as_float((x + 127) << 23);  // normal: the exponent field alone
    return x >= -149 ? __int_as_float(1 << (x + 149)) : 0.0f;  // subnormal: one mantissa bit
}

__device__ __forceinline__ void load_smem_model(SmemModel& S, const DevModel& m) {
    for (int i = threadIdx.x; i < m.C * WP_TRI; i += blockDim.x) {
        int c = i / WP_TRI, k = i % WP_TRI;
        S.dud[c][k] = m.dud[c][k];
        S.bleach[c][k] = m.bleach[c][k];
    }
    for (int t = threadIdx.x; t < m.T; t += blockDim.x) S.p_det[t] = m.p_det[t];
    for (int i = threadIdx.x; i < 16 * 17; i += blockDim.x) {
        const int n = i / 17, tot = i % 17;
        const float qf = 1.0f - m.pf;
        float2 v = make_float2(qf, 0.0f);
        if (tot > 15) {
            v = make_float2(0.0f, 0.0f);  // padding, never read
        } else if (tot > 0) {
            const float c1 = qf * __frcp_rn((float)tot);
            v.x = n < tot ? fmaf(-(float)n, c1, qf) : 0.0f;
            v.y = (float)(n + 1) * c1;
        }
        S.edx[i] = v.x;
        S.edy[i] = v.y;
    }
}

// Arguments of one Baum-Welch E-step (wp_fit.cu).
struct FitArgs {
    const DevModel* model;
    const double* rads;     // [R][T][C]
    int R;
    int D[WP_MAX_CHANNELS];  // dyes per channel of the dye-seq
    int8_t dye[WP_MAX_TIMESTEPS];
    uint8_t tot[WP_MAX_TIMESTEPS];
    const EmitEntry* tab;  // [R][T][C][W] emission factors (non-interacting)
    int W;
    float* scratch;        // per-thread state vectors, interleaved
    long vec_floats;       // floats of one full vector (A and B of T*S states)
    double* sums;          // [nthreads][nslots]
    double* logp;          // [R] log P per read (nullable)
    int nslots;
    int emission;           // also gather the emission statistics (slots fs_emis)
    // Batched EM instances (bootstrap rounds): model[i] is instance i's
    // model, CTAs [i * inst_ctas, (i + 1) * inst_ctas) serve it, and its R
    // reads are read_idx[i * R .. (i + 1) * R) (indices into rads / tab);
    // logp is then per (instance, read).  inst_ctas 0: one instance, reads 0..R-1.
    int inst_ctas;
    const int* read_idx;
};

// ---- kNN stage (wp_nn.cu) -------------------------------------------------
struct NNArgs {
    const float* queries;   // [R][DP]
    int R;                  // queries in this launch (chunk)
    int q0;                 // first query index of the chunk (into per-query arrays)
    const float* coords;    // [N][DP]
    const float* enorm;     // [N] squared norm of each entry's coordinates
    const float* tlo;       // [N / 32 rounded up][DP] per tile of 32 entries: smallest
    const float* thi;       //   and largest coordinate, and the tile's hits
    const int* ttot;
    const int* hits;        // [N] total hits per entry
    int N;
    long long k;
    int* qbin;              // per query (indexed by q0 + local): bin b*
    int* qbelow;            // hits in bins < b*
    long long* qcap;        // hits in bins <= b* (>= entries there)
    const long long* qoff;  // candidate list offset (chunk-relative)
    int* cand_idx;
    float* cand_d2;
    int* cand_hits;         // the entry's hits, next to its index
    unsigned char* cand_bin;  // the distance bin the histogram counted it in
    int* err;
    int slices;             // entry slices (blockIdx.y)
    int slice_len;
    unsigned* shist;        // [slices][R_all][NB] per-slice histograms
    int R_all;              // queries in the whole batch
    long long* sliceoff;    // [slices][R_all] offset of slice s inside query q's list
    long long* slicecap;    // [slices][R_all] room for slice s (its hits in bins <= b*)
    long long* slicecnt;    // [slices][R_all] candidates slice s wrote
    int* qbase;             // [R_all] per query: float bits >> 19 where its bin 1 starts
    const int* slots;       // histogram / threshold over these R queries (null: 0..R-1)
    int sub;                // histogram: CTAs per entry slice (> 1: each covers a
                            // part and adds its counts to shist, zeroed first)
    unsigned char* stmin;   // [R_all][n_super] smallest bin of each read's entries per
    int n_super;            // super-tile (1,024 entries from its slice's start;
                            // n_super = slices x super-tiles per slice)
    const int* sample;      // [sample_n] entries drawn in proportion to their hits
    int sample_n;
    long long hits_total;   // hits over all entries
    // The reference's k-hit set: per query (q0 + local) the final top's
    // squared distance and flags (NNSelectArgs); the threshold then places
    // b* at the bin holding that distance instead of the k-th hit.
    const double* tf_d;
    const int* tf_flag;
};

struct NNSelectArgs {
    int R;                      // queries in this chunk
    int q0;
    const int* qperm;           // [R_all] read index of each (sorted) query slot
    const int* qbin;
    const int* qbase;           // per query bin origin (as NNArgs)
    const int* qbelow;
    int slices;
    int R_all;
    const long long* sliceoff;  // [slices][R_all]
    const long long* slicecnt;  // [slices][R_all]
    const long long* slicecap;  // [slices][R_all] (bounds slicecnt)
    const long long* qoff;
    const int* cand_idx;
    const float* cand_d2;
    const int* cand_hits;
    const unsigned char* cand_bin;
    const int* hits;            // [N]
    const int* src_off;         // [N + 1]
    const int* src_dense;       // [S] dense id
    const double* src_ratio;    // [S] hits / count
    const int* src_hits;        // [S]
    const int* dense_id;        // [U] original id
    const int* dense_pep;       // [U] peptide index (hybrid), may be null
    const int* dense_count;     // [U] peptide count (hybrid), may be null
    int U;
    long long k;
    float inv_two_sig_sq;
    int h;
    double* acc;                // [warps][U] zero on entry, zero on exit
    int* mark;                  // [warps][U]
    int* touched;               // [warps][U]
    int* out_ncand;             // outputs, indexed by q0 + local
    int* out_cand_id;           // [R][h] original ids
    int* out_cand_pep;          // [R][h] peptide indices (may be null)
    double* out_cand_score;     // [R][h]
    double* out_total;
    double* out_subfrac;        // may be null
    // The reference's k-hit set (KNN_KDTREE): per query slot the final top
    // of the kd-tree search's KBest (wp_kbest.cu); an entry is kept iff its
    // (FP64 squared distance, tree position) is at most (tf_d, tf_pos).
    // Null: the shortest distance-ordered prefix reaching k hits.
    const double* tf_d;         // [R_all]
    const int* tf_pos;
    const int* tf_flag;         // bit 0: every entry kept
    const double* rads;         // [reads][TC] FP64 queries (read order); with
                                // them the near entries' weights use FP64
                                // distances
    double two_sig_sq;          // 2 sig^2
    int TC, C, DP, NC;
    const uint8_t* cnt;         // [N][DP] counts per coordinate (tree order)
    const double* ctab;         // [C][NC] coordinate of count n on channel c
    const double* ecoord;       // [N][TC] FP64 coordinates (interacting models), or null
};

// ---- the reference's k-hit set (wp_kbest.cu) ------------------------------
// One kept entry of the replayed KBest: squared distance, tree position and
// hits.
struct KBItem {
    double d;
    int pos;
    int hits;
};

struct KBArgs {
    int nwork;                  // query slots to process
    const int* work;            // their indices (null: 0 .. nwork-1)
    int* next;                  // work counter, zero on entry
    const int* qperm;           // read index of each slot (null: identity)
    const double* rads;         // [reads][TC] FP64 queries
    int TC, C, DP, N;
    long long k;
    const uint8_t* cnt;         // [N][DP] counts (tree order)
    const double* ctab;         // [C][NC] coordinate of count n
    int NC;
    int interact;               // coordinates depend on other channels' counts:
    const double* ecoord;       //   [N][TC] FP64 coordinates
    const float* coords32;      //   [N][DP] FP32 coordinates
    const float* tlo;           // [tiles][DP] per 32 tree positions: box
    const float* thi;
    const float* llo;           // [nodes][DP] per leaf: box
    const float* lhi;
    const int* hits;            // [N] hits per entry (tree order)
    const KDNode* nodes;        // nodes[0] the root
    int stack_cap;              // deepest level + 1
    KBItem* reg;                // per warp: two regions of regcap entries
    int* prev;                  // per warp: two regions of regcap / 16 links
    KBItem* stage;              // per warp: stagecap entries
    int regcap, stagecap;
    double* tf_d;               // per slot: the final top
    int* tf_pos;
    int* tf_flag;               // 1 every entry kept, 2 a refused entry tied
                                // the final top's distance, 4 scratch too small
};

// FP64 squared distance from a query to entry p as LeafNode::consider sums
// it (kd-tree/leaf-node.h:31-62): per coordinate x = q - e, x * x, summed in
// groups of four while i < D - 3, then singly.  Coordinates from the count
// table (ctab[c][n], non-interacting models) or from ecoord.
__device__ __forceinline__ double wp_nn_exact_d2(const double* q64, long p, int TC, int C, int DP,
                                                 const uint8_t* cnt, const double* ctab, int NC,
                                                 const double* ecoord) {
    double acc = 0.0;
    int i = 0;
    const uint8_t* row = cnt + p * DP;
    const double* e = ecoord ? ecoord + p * TC : nullptr;
    for (; i + 3 < TC; i += 4) {
        double t[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const double ev = e ? e[i + u] : ctab[((i + u) % C) * NC + row[i + u]];
            const double x = __dsub_rn(q64[i + u], ev);
            t[u] = __dmul_rn(x, x);
        }
        acc = __dadd_rn(acc, __dadd_rn(__dadd_rn(__dadd_rn(t[0], t[1]), t[2]), t[3]));
    }
    for (; i < TC; i++) {
        const double ev = e ? e[i] : ctab[(i % C) * NC + row[i]];
        const double x = __dsub_rn(q64[i], ev);
        acc = __dadd_rn(acc, __dmul_rn(x, x));
    }
    return acc;
}

// ---- read simulator (wp_sim.cu) -------------------------------------------
// Event probabilities are 33-bit thresholds: an event with probability p
// happens when a uniform 32-bit draw u satisfies u < ceil(p * 2^32), i.e.
// u / 2^32 < p as bernoulli_distribution tests a uniform in [0, 1).
struct SimParams {
    int T, C, P, R;
    unsigned long long seed;
    unsigned long long thr_fail, thr_initial_block, thr_cyclic_block;
    unsigned long long thr_detach[WP_MAX_TIMESTEPS];
    unsigned long long thr_dud[WP_MAX_CHANNELS], thr_bleach[WP_MAX_CHANNELS];
    const DevModel* model;     // emission model
    const int8_t* seqs;        // ragged dye-seqs (channel or -1)
    const int* offsets;        // [P + 1]
    const double* cum;         // [P] cumulative peptide counts (last = total)
    float* rads_f;             // [R][T*C] or null
    double* rads_d;            // [R][T*C] or null
    int* pep;                  // [R] peptide index or -1
    uint8_t* tracks;           // [R][T*C] or null
    int per_peptide;           // > 0: instance r is a dye-track of the peptide
                               // holding copy r / per_peptide (in the order
                               // of the counts), as generate_dye_tracks
                               // enumerates them; 0: peptide drawn by count
};

// ---- dye-track dedup (wp_dedup.cu) ----------------------------------------
// n dye-track instances are packed into W 64-bit words each, stored word-
// major ([W][n]): count j of the track (j = t * C + c) is a field of `bits`
// bits at position j % k of word j / k (k = 64 / bits fields per word, the
// first field most significant), so that comparing the words in order
// compares the tracks lexicographically.  When the source ids span few
// enough values, their offsets ride in the last word's spare low bits, so
// that sorting that word also sorts by id.
struct DedupArgs {
    int n, TC, bits, W;
    int drop_zero;             // leave out the all-zero track
    int fold_id;               // the source id's offset from id_min sits in
    int id_shift;              // the last word's spare low bits at id_shift
    long long id_min;          // (else a separate sort by id)
    uint64_t last_mask;        // the field bits of the last word
    const uint8_t* in_u8;      // [n][TC] instance tracks, or
    const int16_t* in_i16;     // [n][TC] (exactly one of the two)
    const int* pep;            // [n] peptide index (-1: none), or null when
    const int* pep_ids;        //     inst_id / inst_cnt are given
    const int* pep_cnts;
    int* inst_id;              // [n] source id / count of each instance
    int* inst_cnt;
    uint64_t* words;           // [W][n]
    uint64_t* keys0;           // [n] sort keys (ping-pong)
    uint64_t* keys1;
    int* perm0;                // [n] instance order (ping-pong)
    int* perm1;
    int* flag_t;               // [n] first instance of a track / of a source
    int* flag_s;
    int* scan_t;               // [n] inclusive sums of the flags
    int* scan_s;
    int* start;                // [n] first sorted position of each source
    void* temp;                // CUB scratch
    size_t temp_bytes;
    int16_t* out_counts;       // [n][TC] distinct tracks (first U rows)
    int* out_src_off;          // [n + 1]
    int* out_src_id;           // [n] (first S entries)
    int* out_src_count;
    int* out_src_hits;
    int* out_sizes;            // [2]: U, S
};
