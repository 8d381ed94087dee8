/*
 * whatprot_gb300.h -- C ABI of the GB300 (sm_103a) peptide-HMM engine.
 *
 * This is the drop-in boundary for whatprot's classification and fitting hot
 * path.  Plain C types only: callers own every buffer they pass; nothing here
 * throws; every call returns a wp_status.  One wp_ctx per host thread (calls
 * on one context are serialised by an internal mutex).
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the reference project's cc_code/src/).
 */
#ifndef WHATPROT_GB300_H
#define WHATPROT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int wp_status;
enum {
    WP_OK = 0,
    WP_ERR_INVALID = 1,     /* bad argument (null pointer, size out of range) */
    WP_ERR_OOM = 2,         /* device or host allocation failed */
    WP_ERR_CUDA = 3,        /* a CUDA call failed; see wp_last_error */
    WP_ERR_TIMEOUT = 4,     /* a bounded device wait expired */
    WP_ERR_UNSUPPORTED = 5, /* shape beyond this build's limits */
    WP_ERR_STATE = 6        /* model or peptides not uploaded yet */
};

/* Limits of this build (checked; WP_ERR_UNSUPPORTED beyond them). */
#define WP_MAX_CHANNELS 4
#define WP_MAX_TIMESTEPS 64
#define WP_MAX_DYES_PER_CHANNEL 15

typedef struct wp_ctx wp_ctx;

/* Sequencing model, already divided by mu (SequencingModel::with_mu_as_one,
 * parameterization/model/sequencing-model.cc:140-151).  Per-channel arrays
 * have num_channels entries; interactions / flat_interactions are
 * [num_channels][num_channels] row-major: row c is channel c's model, entry o
 * the multiplicative factor for dyes on channel o (1.0 = none), as
 * ChannelModel::interactions / flat_interactions (channel-model.h:35-54).
 * Either interaction pointer may be NULL (all 1.0). */
typedef struct {
    int num_channels;
    double p_edman_failure;
    double p_detach;               /* DecayingRateModel base    */
    double p_initial_detach;       /* DecayingRateModel initial */
    double p_initial_detach_decay; /* DecayingRateModel initial_decay */
    double p_initial_block;
    double p_cyclic_block;
    const double* p_bleach;
    const double* p_dud;
    const double* bg_sig;
    const double* mu;
    const double* sig;
    const double* interactions;
    const double* flat_interactions;
} wp_seq_model;

/* Baum-Welch expected counts of one E-step, the fields of
 * SequencingModelFitter (parameterization/fit/sequencing-model-fitter.h):
 * numerator/denominator per fitted parameter, detach per timestep. */
typedef struct {
    double p_edman_failure_num, p_edman_failure_den;
    double p_detach_x[WP_MAX_TIMESTEPS], p_detach_n[WP_MAX_TIMESTEPS];
    double p_initial_block_num, p_initial_block_den;
    double p_cyclic_block_num, p_cyclic_block_den;
    double p_bleach_num[WP_MAX_CHANNELS], p_bleach_den[WP_MAX_CHANNELS];
    double p_dud_num[WP_MAX_CHANNELS], p_dud_den[WP_MAX_CHANNELS];
} wp_fit_sums;

/* Context on one CUDA device.  Replaces nothing in the reference (which has
 * no device); it owns the stream, the uploaded model and peptide tables. */
wp_status wp_ctx_create(wp_ctx** out, int device);
void wp_ctx_destroy(wp_ctx* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* wp_last_error(const wp_ctx* ctx);

/* Upload the model for num_timesteps.  Replaces the model part of
 * UniversalPrecomputations (hmm/precomputations/universal-precomputations.cc:
 * 23-59: binomial dud/bleach tables, per-timestep detach rates) and the
 * SequencingModel the classifier holds (classifiers/hmm-classifier.h:32-37). */
wp_status wp_model_upload(wp_ctx* ctx, const wp_seq_model* model,
                          int num_timesteps);

/* Upload the peptide (dye-seq) set.  Replaces DyeSeqPrecomputations per
 * dye-seq (hmm/precomputations/dye-seq-precomputations.cc:20-39) and the
 * HMMClassifier's dye_seqs / max_num_dyes (classifiers/hmm-classifier.cc:
 * 35-67).  dye_seqs is ragged: peptide i is dye_seqs[offsets[i] ..
 * offsets[i+1]), entries -1 (unlabeled) or a channel index, trailing -1
 * already trimmed or not (trimming does not change results).  ids[i] is the
 * peptide id written to predictions, counts[i] its multiplicity. */
wp_status wp_peptides_upload(wp_ctx* ctx, const int16_t* dye_seqs,
                             const int32_t* offsets, const int32_t* ids,
                             const int32_t* counts, int num_peptides);

/* Classify reads.  Replaces HMMClassifier::classify(vector<Radiometry>)
 * (classifiers/hmm-classifier.cc:84-93) and, with candidates,
 * HMMClassifier::classify(radiometry, candidate_indices) (:79-82).
 * rads: [num_reads][T][C] host doubles, already divided by mu
 * (io/radiometries-io.cc:50-51).  dist_cutoff is SequencingSettings::
 * dist_cutoff (DBL_MAX: no pruning).  cand / cand_off: optional ragged
 * candidate peptide indices per read (cand_off has num_reads+1 entries);
 * NULL means all peptides.  Outputs per read: id of the best peptide (first
 * in candidate order on ties), its probability and the count-weighted total,
 * with the reference's NaN patch (classifiers/hmm-classifier.h:73-76).  When
 * the best probability is below the double range, score and total are both
 * scaled by the same power of two so that score/total stays exact.
 * out_log_score (nullable) receives log(P_best). */
wp_status wp_hmm_classify(wp_ctx* ctx, const double* rads, int num_reads,
                          double dist_cutoff, const int32_t* cand,
                          const int32_t* cand_off, int32_t* out_id,
                          double* out_score, double* out_total,
                          double* out_log_score);

/* Same as wp_hmm_classify with inputs and outputs already in device memory
 * (d_rads: [num_reads][T][C] doubles; d_cand/d_cand_off as above or NULL;
 * outputs device arrays).  Runs on the context's stream; returns after the
 * launches are queued when `async` is nonzero, else after completion. */
wp_status wp_hmm_classify_device(wp_ctx* ctx, const double* d_rads,
                                 int num_reads, double dist_cutoff,
                                 int32_t* d_out_id, double* d_out_score,
                                 double* d_out_total, int async);

/* Launch sequence of wp_hmm_classify_device captured in a CUDA graph: the
 * second call with the same arguments (reads and output pointers, size,
 * cutoff, model and peptides) captures it, later ones replay it.  On by
 * default; not used while per-kernel timing is enabled. */
wp_status wp_ctx_set_graphs(wp_ctx* ctx, int enable);

/* Engine launch shapes {pass-1 threads, pass-1 CTAs per SM, pass-2 threads,
 * pass-2 CTAs per SM} (threads a multiple of 32 up to 256, CTAs 1..4); NULL
 * returns to the tuned or default shapes.  Results do not depend on them. */
wp_status wp_set_engine_config(wp_ctx* ctx, const int32_t* cfg4);

/* Autotuner: times the classify of a sample of reads ([R][T][C] host,
 * divided by mu) under every feasible engine launch shape and keeps the
 * fastest for this context's shape key (channels, blocking, max dyes,
 * timesteps); later batches with that key use it.  Writes the chosen shape
 * (cfg4, nullable) and its time in ms. */
wp_status wp_autotune(wp_ctx* ctx, const double* rads, int num_reads,
                      double dist_cutoff, int32_t* out_cfg4,
                      double* out_best_ms);

/* log P for every (read, peptide) pair: out_logp[r * P + p] (host), -inf
 * where P == 0.  PeptideHMM::probability (hmm/hmm/peptide-hmm.cc:94-100),
 * per pair, computed in FP32 with exact power-of-two rescaling. */
wp_status wp_hmm_loglik_all(wp_ctx* ctx, const double* rads, int num_reads,
                            double dist_cutoff, double* out_logp);

/* Algorithmic work of the pruned schedule: the number of visited-state
 * operations the reference's pruned step chain performs for every (read,
 * peptide) pair of this batch (emission 1, detach 2, binomial 2 per
 * multiply-add, Edman 6, block 3 when its rate is nonzero, rescale 2 per
 * state per timestep), summed.  Device-computed from the closed-form boxes. */
wp_status wp_hmm_count_flops(wp_ctx* ctx, const double* rads, int num_reads,
                             double dist_cutoff, double* out_flops);

/* Stage a Baum-Welch fit: the dye-seq being fitted (-1 unlabeled, channel
 * index otherwise) and the reads, [num_reads][T][C] host doubles divided by
 * mu.  Replaces the data HMMFitter holds (fitters/hmm-fitter.h:35-48, 118-144:
 * dye_seq, radiometries).  The reads stay on the device until the next
 * wp_fit_begin or the context's destruction. */
wp_status wp_fit_begin(wp_ctx* ctx, const int16_t* dye_seq, int length,
                       const double* rads, int num_reads);

/* One E-step with the context's current model (wp_model_upload): the
 * expected counts of GenericHMM::improve_fit (hmm/hmm/generic-hmm.h:60-109)
 * summed over every staged read, as HMMFitter::fit accumulates them
 * (fitters/hmm-fitter.h:63-78), without pruning (main/run-fit.cc:59).
 * Reads with P == 0 add nothing (generic-hmm.h:85-87) and are counted in
 * *num_zero.  *sum_logp receives the sum of log P over the other reads
 * (HMMFitter::log_likelihood, fitters/hmm-fitter.h:119-142).  Any output
 * pointer but `out` may be NULL.  The dye-seq must have at most 15 dyes per
 * channel and the model no channel interactions (WP_ERR_UNSUPPORTED). */
wp_status wp_fit_estep(wp_ctx* ctx, wp_fit_sums* out, double* sum_logp,
                       int* num_zero);

/* Batched EM instances: one E-step for each of B models over its own list
 * of num_reads staged reads (read_idx [B][num_reads], indices into the
 * reads given to wp_fit_begin, repeats allowed), all in one launch -- the
 * rounds of bootstrap_fit (fitters/bootstrap-fit.cc:37-93), which the
 * reference fits one after another.  The models share the staged fit's
 * channels, timesteps and emission parameters (mu, sig, bg_sig) and have no
 * interactions; emission fitting must be off.  out [B]; sum_logp and
 * num_zero [B] (nullable) as wp_fit_estep's.  The context's current model
 * becomes models[0]. */
wp_status wp_fit_estep_batch(wp_ctx* ctx, const wp_seq_model* models, int B,
                             const int32_t* read_idx, int num_reads,
                             wp_fit_sums* out, double* sum_logp, int* num_zero);

/* E-step kernel choice: 0 (default) one CTA per read with its vectors in
 * shared memory when they fit, else one thread per read; 1 always one
 * thread per read (tests compare the two).  No reference counterpart. */
wp_status wp_fit_set_kernel(wp_ctx* ctx, int kind);

/* Which parameters a fit holds at their starting values: FitSettings and
 * ChannelFitSettings (parameterization/settings/fit-settings.h,
 * channel-fit-settings.h).  Non-zero = hold. */
typedef struct {
    int hold_p_edman_failure;
    int hold_p_detach;
    int hold_p_initial_detach;
    int hold_p_initial_detach_decay;
    int hold_p_initial_block;
    int hold_p_cyclic_block;
    int hold_p_bleach[WP_MAX_CHANNELS];
    int hold_p_dud[WP_MAX_CHANNELS];
    /* Non-zero: also fit each channel's mu, sig and bg_sig from the E-step's
     * emission statistics (wp_fit_emission_mstep).  No reference
     * counterpart: the reference never fits them (fitters/hmm-fitter.cc:
     * 94-95, peptide-emission.h:47-54); 0 keeps its behaviour. */
    int fit_emission;
} wp_fit_settings;

/* The fitted parameters of a SequencingModel.  The reference fits the rates
 * only (bg_sig, mu, sig and the interactions are never fitted:
 * fitters/hmm-fitter.cc:94-95); mu, sig and bg_sig change here only under
 * wp_fit_settings.fit_emission and are otherwise the starting model's. */
typedef struct {
    double p_edman_failure;
    double p_detach;
    double p_initial_detach;
    double p_initial_detach_decay;
    double p_initial_block;
    double p_cyclic_block;
    double p_bleach[WP_MAX_CHANNELS];
    double p_dud[WP_MAX_CHANNELS];
    double mu[WP_MAX_CHANNELS];
    double sig[WP_MAX_CHANNELS];
    double bg_sig[WP_MAX_CHANNELS];
} wp_fit_params;

/* Emission statistics of one E-step: per channel c and dye count n, the
 * posterior weight w of "channel c shows n live dyes" at an emission,
 * summed over reads and timesteps (the detached state shows 0 on every
 * channel), and that weight times the intensity (x) and its square (xx).
 * No reference counterpart (PeptideEmission's improve_fit is a no-op,
 * hmm/step/peptide-emission.cc:255-260). */
typedef struct {
    double w[WP_MAX_CHANNELS][WP_MAX_DYES_PER_CHANNEL + 1];
    double x[WP_MAX_CHANNELS][WP_MAX_DYES_PER_CHANNEL + 1];
    double xx[WP_MAX_CHANNELS][WP_MAX_DYES_PER_CHANNEL + 1];
} wp_emission_sums;

/* Non-zero: the following wp_fit_estep calls also gather the emission
 * statistics (read them with wp_fit_emission_sums). */
wp_status wp_fit_set_emission(wp_ctx* ctx, int enable);

/* The emission statistics of the last wp_fit_estep (zeros when it did not
 * gather them). */
wp_status wp_fit_emission_sums(wp_ctx* ctx, wp_emission_sums* out);

/* Emission M-step, per channel: the mu, sig and bg_sig that maximise the
 * expected log-likelihood of the intensities under ChannelModel's
 * N(mu n, bg_sig^2 + mu n sig^2) (channel-model.h:35-70, no interactions)
 * given the statistics: sum_n [-w_n/2 log v_n - (xx_n - 2 m_n x_n +
 * m_n^2 w_n) / (2 v_n)], m_n = mu n, v_n = bg_sig^2 + mu n sig^2.  Solved
 * by damped Newton in the logarithms of the three parameters from the
 * current values; a channel without weight at n >= 1 fits bg_sig only.
 * Copies every other field of *cur into *next; *step_size (nullable)
 * receives the largest change of the three parameters over the channels. */
wp_status wp_fit_emission_mstep(const wp_emission_sums* sums, int num_channels, const wp_fit_params* cur,
                                wp_fit_params* next, double* step_size);

/* HMMFitter::fit (fitters/hmm-fitter.h:49-117) with its log_likelihood
 * (:119-142): Baum-Welch from `start` on one dye-seq and R reads
 * ([R][T][C] host doubles divided by mu), GPU E-steps (wp_fit_estep), the
 * dud hidden-count correction and the M-step on the host; stops when the
 * largest parameter change is below stopping_threshold or after max_runtime
 * seconds of wall time.  settings may be NULL (fit everything).  Writes the
 * fitted parameters, the last step size, the final log-likelihood (-inf if
 * some read has P == 0 under the fitted model, as log(0) in the reference)
 * and the number of E-steps (iterations may be NULL).  Stages the reads with
 * wp_fit_begin and leaves the fitted model uploaded on the context. */
wp_status wp_hmm_fit(wp_ctx* ctx, const wp_seq_model* start, int num_timesteps,
                     const int16_t* dye_seq, int length, const double* rads,
                     int num_reads, const wp_fit_settings* settings,
                     double stopping_threshold, double max_runtime,
                     wp_fit_params* out, double* step_size, double* log_l,
                     int* iterations);

/* One M-step of HMMFitter::fit (fitters/hmm-fitter.h:80-116) from E-step
 * sums: the dud hidden-count correction for num_reads reads, p = num/den,
 * the detach curve (wp_fit_offset_exponential), holds (settings may be
 * NULL), and the step size (SequencingModel::distance).  Host only: a
 * caller that shards the reads over GPUs adds the shards' wp_fit_estep sums
 * (an all-reduce) and every rank takes the same step. */
wp_status wp_fit_mstep(const wp_fit_sums* sums, int num_channels,
                       int num_timesteps, const int16_t* dye_seq, int length,
                       long long num_reads, const wp_fit_params* current,
                       const wp_fit_settings* settings, wp_fit_params* next,
                       double* step_size);

/* B fits at once (as wp_hmm_fit each, from the same start): instance b
 * fits the reads read_idx[b * reads_each .. (b + 1) * reads_each) (indices
 * into rads [num_reads][T][C], repeats allowed), all instances' E-steps in
 * one launch per iteration (wp_fit_estep_batch) -- bootstrap_fit's rounds
 * (fitters/bootstrap-fit.cc:37-93) as concurrent EM instances.  An instance
 * stops as wp_hmm_fit does; out_params / out_log_ls / out_steps [B]
 * (out_steps nullable).  Emission fitting is not supported here. */
wp_status wp_hmm_fit_batch(wp_ctx* ctx, const wp_seq_model* start, int num_timesteps,
                           const int16_t* dye_seq, int length, const double* rads,
                           int num_reads, const wp_fit_settings* settings,
                           double stopping_threshold, double max_runtime, int B,
                           const int32_t* read_idx, int reads_each,
                           wp_fit_params* out_params, double* out_log_ls,
                           double* out_steps);

/* bootstrap_fit (fitters/bootstrap-fit.cc:37-173): num_rounds fits
 * (wp_hmm_fit) on reads resampled with replacement (indices from a 64-bit
 * Mersenne twister seeded with `seed`; the reference seeds from the clock),
 * run as concurrent EM instances (wp_fit_estep_batch) unless the emission
 * parameters are fitted too (then one after another),
 * one fit on all reads (out_best, its step size and log-likelihood), and
 * per parameter the bounds of the central confidence_interval of the round
 * results (sorted; lower index floor((1-ci)/2 * rounds), upper floor((1 -
 * (1-ci)/2) * rounds), clamped to the last round).  out_rounds /
 * out_log_ls hold num_rounds entries; ci and worst-step outputs may be
 * NULL. */
wp_status wp_hmm_bootstrap_fit(wp_ctx* ctx, const wp_seq_model* start,
                               int num_timesteps, const int16_t* dye_seq,
                               int length, const double* rads, int num_reads,
                               const wp_fit_settings* settings,
                               double stopping_threshold, double max_runtime,
                               int num_rounds, double confidence_interval,
                               unsigned long long seed,
                               wp_fit_params* out_rounds, double* out_log_ls,
                               wp_fit_params* out_best, double* out_step_size,
                               double* out_best_log_l, wp_fit_params* out_ci_min,
                               wp_fit_params* out_ci_max,
                               double* out_worst_round_step);

/* Box-constrained weighted least-squares fit of base + initial *
 * exp(-decay * i), i = 0..n-1, to y with weights w, parameters in [0, 1] and
 * held ones fixed (held[k] != 0), at most 10 Levenberg-Marquardt iterations
 * from params[3] (updated in place).  The detach M-step of
 * DecayingParameterFitter::get (parameterization/fit/decaying-parameter-
 * fitter.cc:42-66) through least_squares_fit_of_offset_exponential
 * (util/levmar-helper.cc:44-85).  Host only. */
wp_status wp_fit_offset_exponential(const double* y, const double* w, int n,
                                    const int* held, double* params);

/* Upload the kNN training set: N unique dye-tracks, counts [N][T][C] (live
 * dyes per timestep and channel), each with sources src_off[e] ..
 * src_off[e+1] of (peptide id, peptide count, hits).  Replaces the
 * dye_tracks vector NNClassifier and HybridClassifier take
 * (classifiers/nn-classifier.cc:100-117, hybrid-classifier.cc:32-51;
 * SourcedData<DyeTrack, SourceCountHitsList<int>>, common/sourced-data.h:
 * 88-140).  Every track needs at least one hit; T * C <= 64.  Entry
 * coordinates follow the context's model (recomputed after wp_model_upload). */
wp_status wp_nn_tracks_upload(wp_ctx* ctx, const int16_t* counts, int num_tracks,
                              int num_timesteps, int num_channels,
                              const int32_t* src_off, const int32_t* src_id,
                              const int32_t* src_count, const int32_t* src_hits);

/* Which k-hit set the kNN stage keeps (wp_nn_classify, wp_hybrid_classify).
 *
 * WP_NN_KDTREE (the default): the reference's.  NNClassifier searches a
 * kd-tree built over the dye-tracks in their upload order
 * (kd-tree/kd-tree.h:36-64, make-node.h:28-80) with a KBest that pops at
 * most one entry per insertion (kd-tree/k-best.h:26-42), so it keeps the
 * tracks within the final farthest kept one, which lies at or beyond the
 * k-th hit.  The library builds the same tree on the host and replays that
 * search on the GPU, so the kept tracks are the reference's.
 *
 * WP_NN_PREFIX: the shortest distance-ordered prefix of the tracks whose
 * hits reach k (no tree search; faster).  It keeps what KBest keeps when
 * tracks arrive nearest first. */
#define WP_NN_KDTREE 0
#define WP_NN_PREFIX 1
wp_status wp_nn_set_selection(wp_ctx* ctx, int selection);

/* The kd-tree NNClassifier builds (KDTree's constructor,
 * kd-tree/kd-tree.h:36-43, make-node.h:28-80) over N entries with
 * coordinates coords [N][D] (D <= 64) for k: writes the input index of the
 * entry at each tree position (perm [N]) and the number of nodes.  Host
 * only; exposed so the build can be checked against the reference's. */
wp_status wp_nn_kd_tree_order(const double* coords, int N, int D, int k, int32_t* perm,
                              int* out_num_nodes);

/* NNClassifier::classify(radiometry, h) (classifiers/nn-classifier.cc:
 * 137-203) for R reads ([R][T][C] host doubles divided by mu): the k-hit
 * nearest dye-tracks (as wp_nn_set_selection picked), Gaussian weights
 * exp(-d^2 / 2 sig^2), per-id scores sum(weight * hits / count), and the
 * top h ids.  Writes per read out_ncand[r] <= h, out_cand_id /
 * out_cand_score [R][h] (ascending score, ties by ascending id; the
 * reference's heap leaves equal scores unordered) and out_total[r] =
 * sum(weight * hits).  h <= 1024. */
wp_status wp_nn_classify(wp_ctx* ctx, const double* rads, int num_reads, int k,
                         double sig, int h, int32_t* out_ncand,
                         int32_t* out_cand_id, double* out_cand_score,
                         double* out_total);

/* HybridClassifier::classify (classifiers/hybrid-classifier.cc:55-94):
 * kNN top-h candidates (as wp_nn_classify), the HMM over those peptides in
 * ascending kNN score (wp_hmm_classify with candidates; ties go to the
 * lowest kNN score), its score multiplied by sum(adjusted kNN score x
 * peptide count), NaN patched.  Peptides come from wp_peptides_upload;
 * candidate ids absent from them map to peptide index 0 with count 0, as in
 * the reference.  A read with no candidate gets (-1, 0, 1). */
wp_status wp_hybrid_classify(wp_ctx* ctx, const double* rads, int num_reads,
                             int k, double sig, int h, double dist_cutoff,
                             int32_t* out_id, double* out_score,
                             double* out_total);

/* wp_hybrid_classify with reads and outputs in device memory (d_rads
 * [num_reads][T][C] doubles; d_out_* device arrays); returns after
 * completion. */
wp_status wp_hybrid_classify_device(wp_ctx* ctx, const double* d_rads,
                                    int num_reads, int k, double sig, int h,
                                    double dist_cutoff, int32_t* d_out_id,
                                    double* d_out_score, double* d_out_total);

/* Simulate reads on the device (simulation/generate-dye-track.cc:29-110,
 * generate-radiometry.cc:28-62): num_reads reads of peptides drawn in
 * proportion to their counts from the uploaded peptide set, with the
 * context's model, counter-based Philox streams from `seed` (read r uses
 * subsequence r).  out_rads [R][T][C] intensities (divided by mu),
 * out_peptide[r] the peptide index, or -1 for a read whose first timestep
 * shows no dye (the reference does not emit those), out_tracks [R][T][C]
 * the live dye counts (may be NULL).  Dye-seqs longer than 256 positions are
 * cut at 256. */
wp_status wp_simulate_reads(wp_ctx* ctx, int num_reads, unsigned long long seed,
                            double* out_rads, int32_t* out_peptide,
                            uint8_t* out_tracks);

/* ---- Dye-track sets (the kNN training data) on the device.  The result of
 * the last of the two calls below stays on the device: wp_dye_tracks_download
 * copies it out, wp_dye_tracks_to_nn makes it the kNN / hybrid training set
 * (as wp_nn_tracks_upload would).  Tracks come out in lexicographic order of
 * their counts and each track's sources in ascending id; the reference's
 * order is that of its hash tables. */

/* dedup_dye_tracks (simulation/dedup-dye-tracks.cc:35-61): num_tracks
 * dye-tracks counts [N][T][C] (non-negative), instance i from source
 * (ids[i], src_counts[i]) -> the distinct tracks, each with one
 * (id, count, hits) per distinct source id: count that of the id's first
 * instance, hits the number of its instances.  All-zero tracks are kept, as
 * the reference keeps them.  Writes the numbers of distinct tracks and of
 * sources. */
wp_status wp_dedup_dye_tracks(wp_ctx* ctx, const int16_t* counts, const int32_t* ids,
                              const int32_t* src_counts, int num_tracks, int T, int C,
                              int* out_num_tracks, int* out_num_sources);

/* generate_dye_tracks (simulation/generate-dye-tracks.cc:32-70) followed by
 * the dedup above, as `simulate dt` runs them (main/run-simulate-dt.cc:
 * 61-81): per_peptide dye-tracks for each of the count copies of every
 * uploaded dye-seq (instance r of copy r / per_peptide, Philox subsequence r
 * of `seed`), the context's model and timesteps; instances with no dye at
 * the first timestep are dropped.  out_instance_tracks [n][T][C] and
 * out_instance_peptide [n] (peptide index, -1 for a dropped instance), n =
 * per_peptide x the sum of the counts, return the instances (may be NULL). */
wp_status wp_simulate_dye_tracks(wp_ctx* ctx, int per_peptide, unsigned long long seed,
                                 int* out_num_tracks, int* out_num_sources,
                                 uint8_t* out_instance_tracks,
                                 int32_t* out_instance_peptide);

/* Copies the last dye-track set out: counts [U][T][C], src_off [U + 1],
 * src_id / src_count / src_hits [S]. */
wp_status wp_dye_tracks_download(wp_ctx* ctx, int16_t* counts, int32_t* src_off,
                                 int32_t* src_id, int32_t* src_count,
                                 int32_t* src_hits);

/* Makes the last dye-track set the kNN / hybrid training set. */
wp_status wp_dye_tracks_to_nn(wp_ctx* ctx);

/* BF16 tensor-core GEMM (tcgen05, TMEM accumulator), the building block of
 * the learned proposal network, exposed for tests: C = act(A . B^T + bias)
 * on device pointers, A [M][K] (pitch lda), B [N][K] (pitch ldb) BF16
 * row-major, K a multiple of 64, pitches multiples of 8; C [M][ldc] FP32
 * (c_fp32) or BF16; bias [N] FP32 or NULL; act 0 none, 1 GELU; Z (BF16
 * pre-activation) or NULL.  Synchronous on the default stream.  No reference
 * counterpart (the reference has no network). */
wp_status wp_dev_gemm_bf16(const void* A, int lda, const void* B, int ldb,
                           int M, int N, int K, void* C, int ldc, int c_fp32,
                           const float* bias, int act, void* Z);

/* ---- Learned proposal network (no reference counterpart).  An MLP from a
 * radiometry (T*C <= 64 intensities, zero padded to 64) to logits over the
 * context's peptides: GELU(W1 x + b1) -> GELU(W2 h + b2) -> W3 h + b3, hidden
 * width `hidden`, BF16 weights and activations, FP32 accumulation on the
 * tensor cores, FP32 master weights and Adam.  It proposes the top-h
 * peptides that the HMM rescores, in place of the kNN stage of the hybrid.
 * A network belongs to the context's device and is tied to the peptide set
 * and read shape it was built for (WP_ERR_STATE otherwise). */
typedef struct wp_mlp wp_mlp;
wp_status wp_mlp_create(wp_ctx* ctx, int hidden, unsigned long long seed,
                        wp_mlp** out);
void wp_mlp_destroy(wp_mlp* mlp);

/* Train on num_reads reads simulated on the device from the context's model
 * and peptides (wp_simulate_reads; fresh reads every step, streams derived
 * from seed), in steps of `batch` (a multiple of 64) with Adam at rate lr.
 * Undetectable reads count as no example.  *out_loss (nullable): the mean
 * cross-entropy of the last step. */
wp_status wp_mlp_train(wp_ctx* ctx, wp_mlp* mlp, long long num_reads, int batch,
                       float lr, unsigned long long seed, double* out_loss);

/* One step on a device batch: d_x [B][T*C] FP32, d_labels [B] peptide
 * indices (-1: skip), B a multiple of 64.  lr 0 computes the gradients only
 * (wp_mlp_get with grad = 1 reads them). */
wp_status wp_mlp_train_step(wp_ctx* ctx, wp_mlp* mlp, const float* d_x,
                            const int32_t* d_labels, int B, float lr,
                            double* out_loss);

/* Parameter tensors: 0 W1 [hidden][64], 1 b1 [hidden], 2 W2 [hidden][hidden],
 * 3 b2, 4 W3 [Ppad][hidden], 5 b3 [Ppad] (Ppad = peptides rounded up to 64;
 * padded rows are zero).  Get copies the FP32 master (grad = 0) or the last
 * gradient (grad = 1) to host; set replaces the master. */
wp_status wp_mlp_shape(const wp_mlp* mlp, int which, long long* rows,
                       long long* cols);
wp_status wp_mlp_get(wp_mlp* mlp, int which, int grad, float* out);
wp_status wp_mlp_set(wp_ctx* ctx, wp_mlp* mlp, int which, const float* in);

/* Logits [R][P] for reads [R][T][C] (host doubles divided by mu). */
wp_status wp_mlp_logits(wp_ctx* ctx, wp_mlp* mlp, const double* rads,
                        int num_reads, float* out);

/* The top h peptides per read: indices [R][h] in ascending logit (ties by
 * index), their softmax probabilities, and (nullable) the candidates'
 * sum of probability x peptide count.  h <= min(1024, peptides). */
wp_status wp_mlp_propose(wp_ctx* ctx, wp_mlp* mlp, const double* rads,
                         int num_reads, int h, int32_t* out_idx,
                         float* out_prob, double* out_mass);

/* The hybrid classifier with the network's proposals in place of the kNN
 * stage: the HMM over the top h peptides (ascending logit; ties go to the
 * lower logit), its score times the candidates' probability mass (sum of
 * softmax probability x count, the analogue of the kNN subfraction), NaN
 * patched. */
wp_status wp_mlp_hybrid_classify(wp_ctx* ctx, wp_mlp* mlp, const double* rads,
                                 int num_reads, int h, double dist_cutoff,
                                 int32_t* out_id, double* out_score,
                                 double* out_total);
wp_status wp_mlp_hybrid_classify_device(wp_ctx* ctx, wp_mlp* mlp,
                                        const double* d_rads, int num_reads,
                                        int h, double dist_cutoff,
                                        int32_t* d_out_id, double* d_out_score,
                                        double* d_out_total);

/* Kernel launches issued by this context since creation (all kinds). */
long long wp_launch_count(const wp_ctx* ctx);

/* Work statistics of the last batch run on this context (synchronises):
 * stats[0] (read, peptide) slots, [1] slots the pruning left non-empty,
 * [2] pairs run by the second engine pass (too large for the first pass's
 * slab), [3] pairs run by the dense fallback.  No reference counterpart. */
wp_status wp_last_batch_stats(wp_ctx* ctx, long long* stats4);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events against it.  No reference counterpart. */
void* wp_ctx_stream(const wp_ctx* ctx);

/* Per-kernel timing with CUDA events recorded on the context's stream around
 * every launch while enabled.  kind: 0 forward (and fit E-step), 1 prep,
 * 2 combine, 3 flop count, 4 kNN distances, 5 kNN select, 6 simulator,
 * 7 dye-track dedup (all its kernels and sorts), 8 kNN kd-tree search
 * replay.  wp_timing_read
 * synchronises and returns the summed duration in ms
 * and the number of launches since the last enable.  No reference
 * counterpart (the reference only prints phase wall times,
 * main/cmd-line-out.cc). */
wp_status wp_timing_enable(wp_ctx* ctx, int enable);
wp_status wp_timing_read(wp_ctx* ctx, int kind, double* total_ms, long long* launches);

/* Runs the engine passes and the dense kernel of the last wp_hmm_classify /
 * wp_hmm_classify_device batch on this context again, `reps` times, on the
 * context's stream (same work lists, the same results written again), and
 * returns their elapsed time in ms.  For measurements of the forward
 * kernels alone (e.g. their DRAM traffic over an interval).  WP_ERR_STATE if
 * no classify batch is held (another kind of call, or a buffer reallocated,
 * since).  No reference counterpart. */
wp_status wp_engine_replay(wp_ctx* ctx, int reps, double* ms);

/* Measured FP32 fused-multiply-add throughput of the context's device in
 * TFLOP/s (2 flops per FMA), from a timed loop of independent FMA chains on
 * every SM.  The denominator of the forward kernel's roofline. */
wp_status wp_probe_fp32_peak(wp_ctx* ctx, double* tflops);

/* Classify without allocating any memory.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc, such as an
 * acquisition loop that may not stall the device with an allocation or a
 * host that runs this library under a memory budget it does not own.  Same
 * kernels and results as wp_hmm_classify (all peptides as candidates), but
 * every input copy and intermediate buffer lives in one device array of
 * 64 MiB that is part of the library (every GPU that loads the library holds
 * it until the process exits); no context, stream or event is created.  All
 * pointers are host pointers; the call runs on the legacy default stream of
 * `device` and returns when the outputs are written.  The first call on a
 * device looks up the array's device address (set-up) and must come before
 * any stream capture.  Inputs whose buffers do not fit the array (32 bytes
 * per (read, peptide) pair plus under 1 KB per read and per peptide: about
 * two million pairs) are rejected with WP_ERR_UNSUPPORTED.  Calls share the array: calls that overlap on the GPU
 * race; calls through this entry point in one process are serialised. */
wp_status wp_hmm_classify_noalloc(int device, const wp_seq_model* model,
                                  int num_timesteps, const int16_t* dye_seqs,
                                  const int32_t* offsets, const int32_t* ids,
                                  const int32_t* counts, int num_peptides,
                                  const double* rads, int num_reads,
                                  double dist_cutoff, int32_t* out_id,
                                  double* out_score, double* out_total);

#ifdef __cplusplus
}
#endif

#endif /* WHATPROT_GB300_H */
