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
#include <stdint.h>

#include "../../include/whatprot_gb300.h"

#define WP_W (WP_MAX_DYES_PER_CHANNEL + 1)      // extent cap per channel
#define WP_TRI (WP_W * (WP_W + 1) / 2)          // triangular table size

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
};

// One peptide.  dye[e] is the channel removed by a successful Edman cycle at
// position e (-1 none), tot[e] = DyeTrack(e, dye[e]).
struct PeptideRec {
    uint8_t D[WP_MAX_CHANNELS];
    int8_t dye[WP_MAX_TIMESTEPS];
    uint8_t tot[WP_MAX_TIMESTEPS];
};

// Emission factor of one table entry: value = mant * 2^expo exactly as the
// reference's FP64 product, mant in [0.5, 1) rounded to FP32; mant == 0 means
// the entry is zero (outside the pruning box, or underflowed in FP64).
struct EmitEntry {
    float mant;
    int expo;
};

#define WP_EXPO_ZERO (-100000)

__host__ __device__ inline int wp_ipow(int b, int e) {
    int r = 1;
    for (int i = 0; i < e; i++) r *= b;
    return r;
}

// Size of one read's slab of emission entries.
__host__ __device__ inline int wp_read_table_entries(int T, int C, int W, int interacting) {
    return interacting ? T * wp_ipow(W, C) : T * C * W;
}

// Arguments of one forward launch (one shape bucket).
struct TileArgs {
    const DevModel* model;
    const PeptideRec* peps;
    const uint8_t* box_lo;   // [R][T][C]
    const uint8_t* box_hi;
    const EmitEntry* table;  // [R][entries]
    int entries;             // per read
    int W;                   // Dmax + 1 (table extent per channel)
    const int* list;         // peptide index per list entry
    const int* key;          // tie-break key (candidate position) per entry
    const int* tile_read;    // per CTA
    const int* tile_begin;
    const int* tile_end;
    const int* tile_out;     // partial index per CTA
    int S_cap;               // max states per Edman slice in this launch
    int num_peptides;
    const int* counts;       // peptide multiplicities
    // outputs
    double* out_logp;        // [R][P] or null
    // per tile partials (classify mode) or null
    int* part_key;
    int* part_pep;
    float* part_mant;
    int* part_expo;
    double* part_total;      // total relative to 2^part_expo
    int* err;                // set nonzero on an internal error
};
