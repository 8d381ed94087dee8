/*
 * wp_oracle.h -- CPU FP64 restatement of whatprot's peptide HMM.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it; the product never links or calls it.
 *
 * It restates, in plain C and double precision, the algorithm of the
 * reference's cc_code/src/hmm/ tree (step chain, KDRange pruning, forward,
 * backward and Baum-Welch expected counts), cc_code/src/parameterization/model
 * (channel model, decaying detach rate) and cc_code/src/classifiers/
 * hmm-classifier.h (argmax + count-weighted total).  Each function cites the
 * reference file:line it follows.  The range pruning is restated literally
 * (prune_forward / prune_backward per step), not in closed form, so that the
 * closed-form boxes used by the CUDA kernels can be checked against it.
 *
 * Parity pin: the five "no change" probabilities of the reference's
 * cc_code/src/hmm/hmm/peptide-hmm.test.cc:188,227,266,305,344 and outputs of
 * the reference itself compiled from source into oracle/_ref (see Makefile).
 */
#ifndef WP_ORACLE_H
#define WP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WPO_MAX_CHANNELS 8
#define WPO_MAX_TIMESTEPS 64

typedef struct {
    int num_channels;
    double p_edman_failure;
    double p_detach;               /* DecayingRateModel.base */
    double p_initial_detach;       /* DecayingRateModel.initial */
    double p_initial_detach_decay; /* DecayingRateModel.initial_decay */
    double p_initial_block;
    double p_cyclic_block;
    double p_bleach[WPO_MAX_CHANNELS];
    double p_dud[WPO_MAX_CHANNELS];
    double bg_sig[WPO_MAX_CHANNELS];
    double mu[WPO_MAX_CHANNELS];
    double sig[WPO_MAX_CHANNELS];
    /* interactions[c][o]: multiplicative factor on channel c's mu per dye on
     * channel o (1.0 = no interaction); flat_interactions likewise, applied
     * once when channel o has any dye (self: when >1 dye). */
    double interactions[WPO_MAX_CHANNELS][WPO_MAX_CHANNELS];
    double flat_interactions[WPO_MAX_CHANNELS][WPO_MAX_CHANNELS];
} wpo_model;

/* Expected counts, one per fitted parameter (SequencingModelFitter). */
typedef struct {
    double edman_num, edman_den;
    double detach_x[WPO_MAX_TIMESTEPS], detach_n[WPO_MAX_TIMESTEPS];
    double init_block_num, init_block_den;
    double cyc_block_num, cyc_block_den;
    double bleach_num[WPO_MAX_CHANNELS], bleach_den[WPO_MAX_CHANNELS];
    double dud_num[WPO_MAX_CHANNELS], dud_den[WPO_MAX_CHANNELS];
    /* Emission statistics (no reference counterpart: PeptideEmission's
     * improve_fit is a no-op, peptide-emission.cc:255-260): per channel c
     * and dye count n, the posterior weight of "channel c shows n live dyes"
     * at an emission, summed over timesteps (the detached state shows 0 on
     * every channel), and that weight times the intensity and its square. */
    double emis_w[WPO_MAX_CHANNELS][16];
    double emis_x[WPO_MAX_CHANNELS][16];
    double emis_xx[WPO_MAX_CHANNELS][16];
} wpo_fit_sums;

/* Channel model (channel-model.h:35-70, channel-model.cc:35-49). */
double wpo_adjusted_mu(const wpo_model* m, int channel, const unsigned* counts);
double wpo_sigma(const wpo_model* m, int channel, double amu);
double wpo_pdf(const wpo_model* m, int channel, double observed,
               const unsigned* counts);
/* DecayingRateModel::operator[] (decaying-rate-model.cc:47-50). */
double wpo_p_detach_at(const wpo_model* m, unsigned t);

/* DyeTrack(T, C, dye_seq) (dye-track.cc:26-43).  out[t*C + c]. */
void wpo_dye_track(int num_timesteps, int num_channels, const int16_t* seq,
                   int length, int16_t* out);

/* PeptideEmission pruned range for one timestep (peptide-emission.cc:50-163).
 * rad is [T][C] (already divided by mu).  Writes [min, max) per channel.
 * dist_cutoff >= DBL_MAX means "no pruning". */
void wpo_emission_range(const wpo_model* m, const double* rad, int t,
                        unsigned max_num_dyes, double dist_cutoff,
                        unsigned* cmin, unsigned* cmax);

/* PeptideHMM(...).probability() for one (radiometry, dye-seq) pair.
 * Returns the reference's FP64 probability.  *log_p receives log(P) computed
 * with exact power-of-two rescaling after every emission (no underflow);
 * *visited_flops receives the visited-state operation count of the pruned
 * schedule (emission 1, detach 2, binomial 2 per MAC, Edman 6, block 3 when
 * p != 0, rescale 2 per state per timestep).  Either pointer may be NULL.
 * max_num_dyes is the classifier-wide Dmax (hmm-classifier.cc:47-66). */
double wpo_peptide_probability(const wpo_model* m, int num_timesteps,
                               const int16_t* seq, int length,
                               const double* rad, unsigned max_num_dyes,
                               double dist_cutoff, double* log_p,
                               double* visited_flops);

/* The pruned ranges of one (radiometry, dye-seq) pair after both prune
 * passes, flattened: for each emission t (0..T-1) the [min,max) per channel
 * of its final pruned_range.  Returns 1 if the pruning emptied the range
 * (probability 0), else 0.  lo/hi are [T][C]. */
int wpo_pruned_emission_boxes(const wpo_model* m, int num_timesteps,
                              const int16_t* seq, int length,
                              const double* rad, unsigned max_num_dyes,
                              double dist_cutoff, unsigned* lo, unsigned* hi);

/* HMMClassifier::classify_helper (hmm-classifier.h:45-78) over a candidate
 * list (all peptides when cand == NULL).  Peptides are given as a ragged
 * array: seqs[offsets[i] .. offsets[i+1]).  Writes the id of the best
 * peptide, its probability and the count-weighted total, with the reference's
 * NaN patch. */
void wpo_classify_one(const wpo_model* m, int num_timesteps,
                      const int16_t* seqs, const int32_t* offsets,
                      const int32_t* ids, const int32_t* counts,
                      int num_peptides, const int32_t* cand, int num_cand,
                      const double* rad, double dist_cutoff, int32_t* out_id,
                      double* out_score, double* out_total);

/* Batch over reads with `threads` worker threads (OpenMP-free, pthreads);
 * rads is [R][T][C].  cand/cand_off may be NULL. */
void wpo_classify_batch(const wpo_model* m, int num_timesteps,
                        const int16_t* seqs, const int32_t* offsets,
                        const int32_t* ids, const int32_t* counts,
                        int num_peptides, const double* rads, int num_reads,
                        const int32_t* cand, const int32_t* cand_off,
                        double dist_cutoff, int threads, int32_t* out_id,
                        double* out_score, double* out_total);

/* log P for every (read, peptide) pair: out[r*P + p]. */
void wpo_loglik_all(const wpo_model* m, int num_timesteps, const int16_t* seqs,
                    const int32_t* offsets, int num_peptides,
                    const double* rads, int num_reads, double dist_cutoff,
                    int threads, double* out_logp);

/* GenericHMM::improve_fit (generic-hmm.h:60-109) for one read: adds this
 * read's expected counts into *sums (when P > 0) and returns P (reference
 * FP64 value); *log_p receives log(P) from the rescaled computation. */
double wpo_improve_fit(const wpo_model* m, int num_timesteps,
                       const int16_t* seq, int length, const double* rad,
                       unsigned max_num_dyes, double dist_cutoff,
                       wpo_fit_sums* sums, double* log_p);
/* The same over R reads [R][T][C] on `threads` host threads (the E-step of
 * one HMMFitter iteration, fitters/hmm-fitter.h:58-78); logp may be NULL. */
void wpo_improve_fit_batch(const wpo_model* m, int T, const int16_t* seq,
                           int length, const double* rads, int R,
                           double dist_cutoff, int threads, wpo_fit_sums* sums,
                           double* logp);

/* KDTEntry coordinates (nn-classifier.cc:59-74): out[(e*T + t)*C + c]. */
void wpo_nn_coords(const wpo_model* m, int T, const int16_t* counts, int N, double* out);

/* The kd-tree of KDTree (kd-tree/kd-tree.h:36-64, make-node.h:28-80) over
 * N entries of D <= 64 coordinates coords [N][D]: pos[i] is the input index
 * of the entry at tree position i (the vector make_node permutes); nodes
 * as make_node creates them (a leaf holds tree positions [begin, end)). */
typedef struct {
    int leaf;
    int s;            /* split dimension */
    int begin, end;   /* leaf: tree positions */
    int left, right;  /* internal: child nodes */
    double max_left, min_right, split;
} wpo_kd_node;

typedef struct {
    int N, D, root, num_nodes, cap;
    wpo_kd_node* nodes;
    int32_t* pos;
} wpo_kd_tree;

int wpo_kd_tree_build(const double* coords, int N, int D, int k, wpo_kd_tree* out);
void wpo_kd_tree_free(wpo_kd_tree* t);
/* KDTree::search: tree_coords [N][D] in tree order, pos_hits[i] the hits of
 * the entry at tree position i; writes the kept tree positions and squared
 * distances farthest first (KBest::fill) and returns their number. */
int wpo_kd_tree_search(const wpo_kd_tree* t, const double* tree_coords, const int* pos_hits,
                       const double* q, int k, int32_t* out_pos, double* out_d2, int max_out);

/* k-hit set selections of the kNN stage */
#define WPO_NN_KDTREE 0 /* the reference's kd-tree search with KBest */
#define WPO_NN_PREFIX 1 /* the shortest distance-ordered prefix */

/* NNClassifier::classify(radiometry, h) (nn-classifier.cc:120-203) for R
 * reads over N dye-tracks (counts [N][T][C], sources CSR src_off[N+1]);
 * writes per read the number of candidates (<= h), their ids and scores in
 * ascending score order ([R][h]) and the total score.  `selection` picks
 * the k-hit set (see wp_oracle.c). */
void wpo_nn_classify_batch(const wpo_model* m, int T, const int16_t* track_counts, int N,
                           const int32_t* src_off, const int32_t* src_id,
                           const int32_t* src_count, const int32_t* src_hits,
                           const double* rads, int R, int k, double sig, int h,
                           int selection, int threads, int32_t* out_ncand, int32_t* out_cand_id,
                           double* out_cand_score, double* out_total);

/* HybridClassifier::classify (hybrid-classifier.cc:55-94) for R reads:
 * the kNN stage above, then the HMM over the candidates (peptides ragged as
 * in wpo_classify_batch). */
void wpo_hybrid_classify_batch(const wpo_model* m, int T, const int16_t* track_counts, int N,
                               const int32_t* src_off, const int32_t* src_id,
                               const int32_t* src_count, const int32_t* src_hits,
                               const int16_t* seqs, const int32_t* offsets, const int32_t* ids,
                               const int32_t* counts, int P, const double* rads, int R, int k,
                               double sig, int h, double dist_cutoff, int selection, int threads,
                               int32_t* out_id, double* out_score, double* out_total);

/* dedup_dye_tracks (simulation/dedup-dye-tracks.cc:35-141): n dye-tracks
 * [n][T][C] with sources (ids[i], cnts[i]) -> the distinct tracks, each with
 * one (id, count, hits) per distinct source id: count is that of the id's
 * first instance (dedup-dye-tracks.cc:119-124), hits the number of
 * instances.  The reference's output order is that of its hash tables; this
 * one is canonical: tracks in lexicographic order of their counts, sources
 * in ascending id.  The out arrays hold at least n tracks and n sources;
 * returns the number of tracks and writes the number of sources. */
int wpo_dedup_dye_tracks(int T, int C, int n, const int16_t* counts, const int32_t* ids,
                         const int32_t* cnts, int16_t* out_counts, int32_t* out_src_off,
                         int32_t* out_src_id, int32_t* out_src_count, int32_t* out_src_hits,
                         int32_t* out_num_sources);

/* `simulate dt` (main/run-simulate-dt.cc:61-81): generate_dye_tracks
 * (simulation/generate-dye-tracks.cc:32-70; per dye-seq, per_peptide tracks
 * for each of its count copies, generate_dye_track, generate-dye-track.cc:
 * 29-110; instances with no dye at t = 0 dropped) from a seeded xoshiro256**
 * stream, then wpo_dedup_dye_tracks.  Single-threaded, as the reference.
 * The out arrays hold per_peptide x sum(counts) tracks and sources; returns
 * the number of distinct tracks, writes the sources and kept instances. */
int wpo_simulate_dt(const wpo_model* m, int T, const int16_t* seqs, const int32_t* offsets,
                    const int32_t* ids, const int32_t* counts, int P, int per_peptide,
                    uint64_t seed, int16_t* out_counts, int32_t* out_src_off,
                    int32_t* out_src_id, int32_t* out_src_count, int32_t* out_src_hits,
                    int32_t* out_num_sources, int32_t* out_instances);

#ifdef __cplusplus
}
#endif

#endif /* WP_ORACLE_H */
