// wp_capi.cu -- host side of the C ABI declared in include/whatprot_gb300.h.
//
// The context owns one CUDA stream and the device copies of the model
// (DevModel) and the peptide set (PeptideRec[]).  One batch of reads runs
// as a fixed sequence of launches on that stream, with no host round trip
// in between:
//   prep      per (read, t): emission pruning boxes and factors
//   summary   per read: closed-form pruning boxes, allow flags, emptiness
//   compact   per read: empty pairs -> probability 0; others -> work list
//   engine    thread-per-pair pruned forward pass, pass 1 (small per-thread
//             shared-memory slabs, many resident warps) and pass 2 (large
//             slabs) on what did not fit
//   dense     warp-per-pair forward pass on what did not fit pass 2
//   reduce    per read: best peptide and weighted total (classify), or
//   logp      log P per pair (all-pairs mode)
// The engine and dense kernels are persistent grids that pull work from
// device-side counters, so the list sizes never travel to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "wp_common.cuh"
#include "wp_kdtree.h"

// Kernels.
__global__ void wp_prep_reads_kernel(const DevModel*, const double*, int, unsigned, double,
                                     uint8_t*, uint8_t*, EmitEntry*, int);
__global__ void wp_read_summary_kernel(BatchArgs);
__global__ void wp_window_factors_kernel(BatchArgs);
size_t wp_window_smem_bytes(int C, int W, int threads);
__global__ void wp_compact_kernel(BatchArgs);
__global__ void wp_compact_groups_kernel(BatchArgs);
size_t wp_compact_groups_smem_bytes(int n_grp, int P);
__global__ void wp_reduce_kernel(BatchArgs, int32_t*, double*, double*, double*, const int*);
__global__ void wp_logp_kernel(const float*, const int*, long, double*);
__global__ void wp_count_flops_kernel(BatchArgs, double*);
cudaError_t wp_launch_engine(int C, bool has_block, int threads, size_t smem, cudaStream_t s,
                             const BatchArgs& a, const int2* in, const int* in_count, int* in_head,
                             int2* out, int* out_count, int slab_half, int scr_floats,
                             int spill_error, int* grid_out);
size_t wp_engine_smem_bytes(int slab_half, int scr_floats, bool has_block, int threads);
cudaError_t wp_launch_dense(bool has_block, int threads, size_t smem, cudaStream_t stream,
                            const BatchArgs& a);
size_t wp_dense_smem_bytes(int T, int S_cap, int C, bool has_block, int warps);
cudaError_t wp_launch_fma_probe(int blocks, int threads, int iters, cudaStream_t stream, float* sink);
cudaError_t wp_launch_fit_estep(bool has_block, int grid, int threads, cudaStream_t s, const FitArgs& a);
cudaError_t wp_launch_nn_dist(int DP, bool hist, cudaStream_t s, const NNArgs& a);
cudaError_t wp_launch_nn_select(int grid, cudaStream_t s, const NNSelectArgs& a);
cudaError_t wp_launch_nn_threshold(cudaStream_t s, const NNArgs& a);
cudaError_t wp_launch_nn_estimate(int DP, cudaStream_t s, const NNArgs& a);
size_t wp_nn_sort_temp_bytes(int R);
cudaError_t wp_launch_nn_redo(const NNArgs& a, int* list, int* count, int shift, cudaStream_t s);
cudaError_t wp_launch_nn_zero_hist(const NNArgs& a, cudaStream_t s);
cudaError_t wp_launch_nn_sort_queries(const float* rows, int R, int DP, int TC, float* sorted, int* perm,
                                      unsigned long long* keys, int* idx, void* temp, size_t temp_bytes,
                                      cudaStream_t s);
int wp_nn_bins();
cudaError_t wp_launch_kbest(int grid, cudaStream_t s, const KBArgs& a);
size_t wp_kbest_smem_bytes(int TC, int NC, int stack_cap, bool inter);
int wp_kbest_warps_per_cta();
int wp_kbest_chunk();
int wp_engine_max_threads();
cudaError_t wp_launch_sim_reads(const SimParams& p, cudaStream_t s);
size_t wp_dedup_temp_bytes(int n);
cudaError_t wp_launch_dedup_range(const int16_t* c, size_t total, int* minmax, cudaStream_t s);
cudaError_t wp_launch_dedup(const DedupArgs& a, cudaStream_t s, int* launches);
#include <cuda_bf16.h>
cudaError_t wp_mlp_launch_input(const float* xf, const double* xd, int B, int TC, __nv_bfloat16* X, cudaStream_t s);
cudaError_t wp_mlp_launch_transpose(const __nv_bfloat16* in, int rows, int cols, int ld_in, __nv_bfloat16* out,
                                    int ld_out, cudaStream_t s);
cudaError_t wp_mlp_launch_softmax_ce(const float* logits, int B, int P, int ld, const int* labels, float scale,
                                     __nv_bfloat16* dL, double* loss, cudaStream_t s);
cudaError_t wp_mlp_launch_gelu_bwd(const float* dH, const __nv_bfloat16* Z, long n, __nv_bfloat16* dZ, cudaStream_t s);
cudaError_t wp_mlp_launch_colsum(const __nv_bfloat16* M, int rows, int cols, int ld, float* out, cudaStream_t s);
cudaError_t wp_mlp_launch_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2,
                               float eps, float bc1, float bc2, __nv_bfloat16* wb, cudaStream_t s);
cudaError_t wp_mlp_launch_to_bf16(const float* in, long n, __nv_bfloat16* out, cudaStream_t s);
cudaError_t wp_mlp_launch_init(float* w, long rows, long cols, long valid_rows, float std, unsigned long long seed,
                               cudaStream_t s);
cudaError_t wp_mlp_launch_topk(const float* logits, int R, int P, int ld, int h, const int* counts, int* idx,
                               float* prob, double* mass, int* fail, cudaStream_t s);
cudaError_t wp_gemm_bf16_tn(const void* A, int lda, const void* B, int ldb, int M, int N, int K, void* C, int ldc,
                            int c_fp32, const float* bias, int act, void* Z, int accumulate, int* err,
                            cudaStream_t s);
cudaError_t wp_launch_nn_queries(const double* rads, int R, int TC, int DP, float* out, cudaStream_t s);
cudaError_t wp_launch_nn_ragged(const int* cand, int h, const int* off, int R, int* out, cudaStream_t s);
cudaError_t wp_launch_hybrid_finish(const int* ncand, const double* subfrac, int R, int* id, double* score,
                                    double* total, cudaStream_t s);
int wp_nn_queries_per_block();
int wp_nn_select_warps();
int wp_nn_hmax();
__global__ void wp_fit_reduce_kernel(const double*, long, int, double*);
int wp_fit_nslots(int T, int C, bool emission);
size_t wp_fit_cta_smem_bytes(int T, int C, int S, bool has_block, bool emission);
long wp_fit_cta_ckpt_floats(int T, int S, bool has_block);
cudaError_t wp_launch_fit_cta(bool has_block, int grid, size_t smem, cudaStream_t s, const FitArgs& a, float* ckpt,
                              long ck_stride);
int wp_fit_cta_ctas_per_sm(bool has_block, size_t smem);
long wp_fit_floats_per_thread(int T, int C, int S, bool has_block);

namespace {

// Incremented whenever a device buffer is (re)allocated: a captured graph
// holds buffer addresses, so it is only replayed while this is unchanged.
long long g_alloc_epoch = 0;

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
        g_alloc_epoch++;
    }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        g_alloc_epoch++;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// Engine pass shapes (threads per CTA).
constexpr int kPass1Threads = 256;
constexpr int kPass2Threads = 256;

}  // namespace

// Launch shape of the two engine passes: threads per CTA and CTAs per SM
// (the slab per thread follows from them), chosen by wp_autotune per
// (channels, blocking, max dyes, timesteps) or the default below.
struct EngineCfg {
    int t1 = 256, s1 = 2, t2 = 256, s2 = 1;
    bool operator==(const EngineCfg& o) const { return t1 == o.t1 && s1 == o.s1 && t2 == o.t2 && s2 == o.s2; }
};

// Arguments a captured classify graph was built for.
struct GraphKey {
    const double* rads = nullptr;
    int R = -1;
    double cutoff = 0;
    void* out[3] = {nullptr, nullptr, nullptr};
    long long model_version = -1, pep_version = -1, alloc_epoch = -1;
    EngineCfg cfg;
    bool operator==(const GraphKey& o) const {
        return rads == o.rads && R == o.R && cutoff == o.cutoff && out[0] == o.out[0] && out[1] == o.out[1] &&
               out[2] == o.out[2] && model_version == o.model_version && pep_version == o.pep_version &&
               alloc_epoch == o.alloc_epoch && cfg == o.cfg;
    }
};

// The engine launches of the last classify batch (wp_engine_replay).
struct EngineReplay {
    bool valid = false;
    long long epoch = -1;  // g_alloc_epoch when recorded
    BatchArgs a;
    int C = 0, T = 0, nt = 0, dense_warps = 0;
    bool hb = false;
    int threads[WP_MAX_TIERS], half[WP_MAX_TIERS];
    int2* list[WP_MAX_TIERS];
    int* cnt = nullptr;
};

struct wp_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    EngineReplay replay;
    std::mutex mu;
    std::string err;
    long long launches = 0;
    int smem_optin = 0;

    bool have_model = false;
    DevModel hm;
    // the model's rates in FP64 (the simulator draws with them)
    double raw_pf = 0, raw_pib = 0, raw_pcb = 0;
    double raw_pdet[WP_MAX_TIMESTEPS] = {0};
    double raw_pdud[WP_MAX_CHANNELS] = {0}, raw_pbleach[WP_MAX_CHANNELS] = {0};
    // peptides as the simulator reads them
    long long sim_pep_version = -1;
    DevBuf d_sim_seqs, d_sim_off, d_sim_cum, d_sim_rads, d_sim_pep, d_sim_tracks, d_sim_ids, d_sim_cnts;
    int sim_max_dyes = 0;  // most dyes of one channel in one peptide
    DevBuf d_model;
    // dye-track dedup (wp_dedup.cu): scratch, and the last result, which
    // stays on the device until downloaded or made the kNN training set
    DevBuf d_dd_in, d_dd_words, d_dd_k0, d_dd_k1, d_dd_p0, d_dd_p1, d_dd_id, d_dd_cnt, d_dd_ft, d_dd_fs, d_dd_st,
            d_dd_ss, d_dd_start, d_dd_temp, d_dd_counts, d_dd_off, d_dd_sid, d_dd_scnt, d_dd_hits, d_dd_sizes;
    bool dd_valid = false;
    int dd_U = 0, dd_S = 0, dd_T = 0, dd_C = 0;

    bool have_peps = false;
    std::vector<int16_t> seqs;
    std::vector<int32_t> offsets, ids, counts;
    int P = 0;
    // Derived at plan time (need C and T).
    int plan_C = -1, plan_T = -1;
    int dmax = 0;
    int S_max = 1;       // max over peptides of prod_c (D_c + 1)
    int scr_floats = 1;  // max over peptides of sum_c (D_c + 1)
    std::vector<PeptideRec> recs;
    DevBuf d_peps, d_ids, d_counts, d_perm, d_shape_rank, d_uniq_D, d_pep_u;
    int n_uniq_D = 0;
    DevBuf d_grp_start, d_grp_D;  // runs of perm with one dye-count vector
    int n_grp = 0;

    // Kernel timing.
    bool timing = false;
    struct Timed {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;
    double t_ms[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long t_n[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    size_t nn_acc_cleared = 0;  // bytes of the kNN accumulators known to be zero

    // engine launch shapes (autotuned per shape key) and classify graphs
    std::vector<std::pair<long long, EngineCfg>> tuned;
    bool force_cfg = false;
    EngineCfg forced;
    bool graphs = true;
    GraphKey gkey, gpending;
    cudaGraphExec_t gexec = nullptr;
    long long graph_launches = 0;  // kernels in the captured graph
    int last_engine_grid = 0;
    long long last_slots = 0;

    // Staged Baum-Welch fit.
    bool have_fit = false;
    bool fit_force_thread = false;  // tests: run the thread-per-read E-step
    bool fit_emission = false;      // E-steps also gather the emission statistics
    wp_emission_sums fit_emis_last{};  // those of the last E-step
    int fit_R = 0, fit_T = 0, fit_C = 0;
    int fit_D[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    int fit_dmax = 0;
    std::vector<int16_t> fit_seq;
    DevBuf d_fit_rads, d_fit_lo, d_fit_hi, d_fit_tab, d_fit_scratch, d_fit_sums, d_fit_out, d_fit_logp;
    DevBuf d_boot_models, d_boot_idx;  // batched EM instances

    // kNN training set (unique dye-tracks with sources).
    long long model_version = 0;
    bool have_tracks = false;
    int nn_N = 0, nn_T = 0, nn_C = 0, nn_U = 0;
    long long nn_hits_total = 0;
    int nn_sample_n = 0;  // entries sampled in proportion to their hits (d_nn_sample)
    long long nn_coords_version = -1;
    long long nn_pep_version = -1;
    long long pep_version = 0;
    std::vector<int16_t> nn_counts;
    std::vector<int32_t> nn_src_off, nn_src_id, nn_src_count, nn_src_hits, nn_uniq;
    DevBuf d_nn_coords, d_nn_hits, d_nn_src_off, d_nn_src_dense, d_nn_src_ratio, d_nn_src_hits, d_nn_dense_id,
            d_nn_dense_pep, d_nn_dense_count, d_nn_queries, d_nn_qbin, d_nn_qbase, d_nn_sample, d_nn_qbelow, d_nn_qcap, d_nn_qoff,
            d_nn_cidx, d_nn_cd2, d_nn_chits, d_nn_cbin, d_nn_enorm, d_nn_tlo, d_nn_thi, d_nn_ttot,
            d_nn_qsorted, d_nn_qperm, d_nn_qkeys, d_nn_qidx, d_nn_qtemp, d_nn_redo, d_nn_stmin, d_nn_acc, d_nn_mark, d_nn_touched, d_nn_ncand, d_nn_cand_id, d_nn_cand_pep,
            d_nn_cand_score, d_nn_total, d_nn_subfrac, d_nn_cand_off, d_nn_cand_flat, d_nn_err, d_nn_shist,
            d_nn_sliceoff, d_nn_slicecap, d_nn_slicecnt;
    // The device arrays above hold the entries in the order of the kd-tree
    // NNClassifier builds for k = nn_tree_k (wp_kdtree.cc): tree position p
    // is input entry nn_perm[p].
    int nn_selection = WP_NN_KDTREE;
    long long nn_tree_k = -1;
    std::vector<int> nn_perm;
    std::vector<KDNode> nn_nodes;
    int nn_depth = 0, nn_NC = 0;
    bool nn_inter = false;
    DevBuf d_nn_cnt8, d_nn_nodes, d_nn_ctab, d_nn_ecoord, d_nn_llo, d_nn_lhi;
    // the replay's scratch and results (wp_kbest.cu)
    DevBuf d_kb_reg, d_kb_prev, d_kb_stage, d_kb_next, d_kb_work, d_kb_tfd, d_kb_tfpos, d_kb_tfflag;

    // Per-batch scratch.
    DevBuf d_rads, d_lo, d_hi, d_Ls, d_Up, d_Lpk, d_Upk, d_allow, d_flags, d_table, d_gtab, d_gdelta, d_gK,
            d_gone,
            d_res_mant, d_res_expo, d_pair_info, d_rd,
            d_work, d_ovf1, d_ovf2, d_ovf3, d_ovf4, d_ovf5, d_counters, d_cand, d_slot_off, d_out_id, d_out_score,
            d_out_total, d_out_log, d_logp, d_flops, d_err;
};

namespace {

wp_status fail(wp_ctx* ctx, wp_status code, const std::string& msg) {
    ctx->err = msg;
    return code;
}

wp_status cuda_fail(wp_ctx* ctx, cudaError_t e, const char* what) {
    ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? WP_ERR_OOM : WP_ERR_CUDA;
}

#define WP_CUDA(call, what)                                     \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what); \
    } while (0)

// Event pair around a launch when timing is enabled.
struct TimedLaunch {
    wp_ctx* ctx;
    int kind;
    cudaEvent_t a = nullptr, b = nullptr;
    TimedLaunch(wp_ctx* c, int k) : ctx(c), kind(k) {
        if (ctx->timing) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, ctx->stream);
        }
    }
    ~TimedLaunch() {
        if (ctx->timing) {
            cudaEventRecord(b, ctx->stream);
            ctx->timed.push_back({kind, a, b});
        }
    }
};

void collect_timing(wp_ctx* ctx) {
    for (auto& t : ctx->timed) {
        float ms = 0.0f;
        cudaEventSynchronize(t.b);
        cudaEventElapsedTime(&ms, t.a, t.b);
        ctx->t_ms[t.kind] += ms;
        ctx->t_n[t.kind] += 1;
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    ctx->timed.clear();
}

// BinomialTransition::reserve (hmm/step/binomial-transition.cc:51-67) in
// FP64, rounded once to FP32.
// Per-peptide records (DyeSeqPrecomputations, dye-seq-precomputations.cc:
// 20-39) for the current (C, T).
wp_status plan_peptides(wp_ctx* ctx) {
    const int C = ctx->hm.C, T = ctx->hm.T;
    if (ctx->plan_C == C && ctx->plan_T == T) return WP_OK;
    const int P = ctx->P;
    ctx->recs.assign(P, PeptideRec());
    ctx->dmax = 0;
    ctx->S_max = 1;
    ctx->scr_floats = 1;
    for (int i = 0; i < P; i++) {
        PeptideRec& rec = ctx->recs[i];
        memset(&rec, 0, sizeof(rec));
        const int16_t* s = ctx->seqs.data() + ctx->offsets[i];
        int len = ctx->offsets[i + 1] - ctx->offsets[i];
        int cnt[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        for (int k = 0; k < len; k++) {
            int d = s[k];
            if (d < -1 || d >= C)
                return fail(ctx, WP_ERR_INVALID, "dye-seq " + std::to_string(i) + " uses channel " +
                                                         std::to_string(d) + " >= num_channels");
            if (d >= 0) cnt[d]++;
        }
        int prod = 1, sum = 0;
        for (int c = 0; c < C; c++) {
            if (cnt[c] > WP_MAX_DYES_PER_CHANNEL)
                return fail(ctx, WP_ERR_UNSUPPORTED, "dye-seq " + std::to_string(i) +
                                                             " has more than 15 dyes on one channel");
            rec.D[c] = (uint8_t)cnt[c];
            ctx->dmax = std::max(ctx->dmax, cnt[c]);
            prod *= cnt[c] + 1;
            sum += cnt[c] + 1;
        }
        ctx->S_max = std::max(ctx->S_max, prod);
        ctx->scr_floats = std::max(ctx->scr_floats, sum);
        // DyeTrack(e, c) for c = dye_seq[e] (common/dye-track.cc:26-43).
        int rem[WP_MAX_CHANNELS];
        memcpy(rem, cnt, sizeof(rem));
        for (int e = 0; e < WP_MAX_TIMESTEPS; e++) {
            int d = e < len ? s[e] : -1;
            rec.dye[e] = (int8_t)d;
            rec.tot[e] = (uint8_t)(d >= 0 ? rem[d] : 0);
            if (d >= 0) rem[d]--;
        }
        wp_pack_peptide(rec);
    }
    // Distinct dye-count vectors (the compaction sizes a pair's boxes once
    // per read and distinct vector) and each peptide's vector.
    {
        std::vector<uint32_t> uniq;
        std::vector<int> pu(P);
        std::unordered_map<uint32_t, int> at;
        for (int i = 0; i < P; i++) {
            uint32_t k = 0;
            for (int c = 0; c < WP_MAX_CHANNELS; c++) k |= (uint32_t)ctx->recs[i].D[c] << (8 * c);
            auto it = at.find(k);
            if (it == at.end()) {
                it = at.emplace(k, (int)uniq.size()).first;
                uniq.push_back(k);
            }
            pu[i] = it->second;
        }
        ctx->n_uniq_D = (int)uniq.size();
        WP_CUDA(ctx->d_uniq_D.ensure(sizeof(uint32_t) * std::max<size_t>(uniq.size(), 1)), "alloc dye-count vectors");
        WP_CUDA(ctx->d_pep_u.ensure(sizeof(int) * std::max(P, 1)), "alloc dye-count vectors");
        WP_CUDA(cudaMemcpyAsync(ctx->d_uniq_D.p, uniq.data(), sizeof(uint32_t) * uniq.size(), cudaMemcpyHostToDevice,
                                ctx->stream), "copy dye-count vectors");
        WP_CUDA(cudaMemcpyAsync(ctx->d_pep_u.p, pu.data(), sizeof(int) * P, cudaMemcpyHostToDevice, ctx->stream),
                "copy dye-count vectors");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    }
    // Shape order (Edman-slice size, then dye counts) for the compaction.
    std::vector<int> perm(P);
    for (int i = 0; i < P; i++) perm[i] = i;
    auto key = [&](int i) {
        long k = 1;
        for (int c = 0; c < C; c++) k *= ctx->recs[i].D[c] + 1;
        for (int c = 0; c < C; c++) k = k * 16 + ctx->recs[i].D[c];
        return k;
    };
    std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return key(x) < key(y); });
    std::vector<int> rank(P);
    for (int i = 0; i < P; i++) rank[perm[i]] = i;
    WP_CUDA(ctx->d_shape_rank.ensure(sizeof(int) * std::max(P, 1)), "alloc shape rank");
    WP_CUDA(cudaMemcpyAsync(ctx->d_shape_rank.p, rank.data(), sizeof(int) * P, cudaMemcpyHostToDevice, ctx->stream),
            "copy shape rank");
    WP_CUDA(ctx->d_perm.ensure(sizeof(int) * std::max(P, 1)), "alloc perm");
    WP_CUDA(cudaMemcpyAsync(ctx->d_perm.p, perm.data(), sizeof(int) * P, cudaMemcpyHostToDevice, ctx->stream),
            "copy perm");
    // Groups: the runs of the shape order with one dye-count vector (the key
    // orders by the vector, so each vector is one run).
    {
        std::vector<int> gs;
        std::vector<uint32_t> gd, pdw(P);
        for (int i = 0; i < P; i++) {
            uint32_t k = 0;
            for (int c = 0; c < WP_MAX_CHANNELS; c++) k |= (uint32_t)ctx->recs[i].D[c] << (8 * c);
            pdw[i] = k;
        }
        for (int i = 0; i < P; i++)
            if (i == 0 || pdw[perm[i]] != pdw[perm[i - 1]]) {
                gs.push_back(i);
                gd.push_back(pdw[perm[i]]);
            }
        gs.push_back(P);
        ctx->n_grp = (int)gd.size();
        WP_CUDA(ctx->d_grp_start.ensure(sizeof(int) * gs.size()), "alloc groups");
        WP_CUDA(ctx->d_grp_D.ensure(sizeof(uint32_t) * std::max<size_t>(gd.size(), 1)), "alloc groups");
        WP_CUDA(cudaMemcpyAsync(ctx->d_grp_start.p, gs.data(), sizeof(int) * gs.size(), cudaMemcpyHostToDevice,
                                ctx->stream), "copy groups");
        if (!gd.empty())
            WP_CUDA(cudaMemcpyAsync(ctx->d_grp_D.p, gd.data(), sizeof(uint32_t) * gd.size(), cudaMemcpyHostToDevice,
                                    ctx->stream), "copy groups");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    }
    WP_CUDA(ctx->d_peps.ensure(sizeof(PeptideRec) * std::max(P, 1)), "alloc peptides");
    WP_CUDA(cudaMemcpyAsync(ctx->d_peps.p, ctx->recs.data(), sizeof(PeptideRec) * P,
                            cudaMemcpyHostToDevice, ctx->stream), "copy peptides");
    WP_CUDA(ctx->d_ids.ensure(sizeof(int) * std::max(P, 1)), "alloc ids");
    WP_CUDA(cudaMemcpyAsync(ctx->d_ids.p, ctx->ids.data(), sizeof(int) * P, cudaMemcpyHostToDevice,
                            ctx->stream), "copy ids");
    WP_CUDA(ctx->d_counts.ensure(sizeof(int) * std::max(P, 1)), "alloc counts");
    WP_CUDA(cudaMemcpyAsync(ctx->d_counts.p, ctx->counts.data(), sizeof(int) * P,
                            cudaMemcpyHostToDevice, ctx->stream), "copy counts");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync plan");
    ctx->plan_C = C;
    ctx->plan_T = T;
    return WP_OK;
}

// Largest slab half (state elements) that lets `per_sm` CTAs of `threads`
// share one SM's shared memory.
int slab_half_for(wp_ctx* ctx, int threads, int per_sm, bool hb) {
    size_t budget = (size_t)ctx->smem_optin;
    if (per_sm > 1) budget = std::min(budget, (size_t)(228 * 1024) / per_sm - 1024);
    size_t elem = hb ? 8 : 4;
    size_t fixed = wp_engine_smem_bytes(0, 0, hb, threads);
    if (budget <= fixed) return 0;
    return (int)((budget - fixed) / (2 * elem * threads));
}

long long cfg_key(const wp_ctx* ctx) {
    return ((long long)ctx->hm.C * 2 + (ctx->hm.has_block ? 1 : 0)) * 100000 + (long long)ctx->dmax * 100 + ctx->hm.T;
}

EngineCfg cfg_for(const wp_ctx* ctx) {
    if (ctx->force_cfg) return ctx->forced;
    const long long k = cfg_key(ctx);
    for (const auto& kv : ctx->tuned)
        if (kv.first == k) return kv.second;
    return EngineCfg();
}

enum Mode { MODE_CLASSIFY, MODE_LOGP, MODE_FLOPS };

// Everything between "reads are on the device" and "per-read outputs are
// on the device".  Slots: all peptides (cand == null) or a ragged candidate
// list per read (host arrays, copied here).
wp_status run_batch(wp_ctx* ctx, const double* d_rads, int R, double dist_cutoff,
                    const int32_t* h_cand, const int32_t* h_cand_off, Mode mode, double* d_logp,
                    int32_t* d_out_id, double* d_out_score, double* d_out_total, double* d_out_log,
                    double* d_flops, const int32_t* d_cand_in = nullptr, const int32_t* d_cand_off_in = nullptr) {
    const int C = ctx->hm.C, T = ctx->hm.T;
    ctx->replay.valid = false;
    wp_status st = plan_peptides(ctx);
    if (st != WP_OK) return st;
    const bool hb = ctx->hm.has_block != 0;
    const int W = ctx->dmax + 1;
    const int entries = wp_read_table_entries(T, C, W, ctx->hm.interacting);
    // Candidates: host lists (h_cand, h_cand_off) or device lists
    // (d_cand_in, d_cand_off_in, with the host copy of the offsets).
    const bool have_cand = h_cand || d_cand_in;
    long n_slots = have_cand ? (long)h_cand_off[R] : (long)R * ctx->P;
    if (n_slots > INT32_MAX) return fail(ctx, WP_ERR_UNSUPPORTED, "too many (read, peptide) pairs in one batch");
    const size_t rtc = (size_t)R * T * C;
    WP_CUDA(ctx->d_lo.ensure(rtc), "alloc");
    WP_CUDA(ctx->d_hi.ensure(rtc), "alloc");
    WP_CUDA(ctx->d_Ls.ensure(rtc), "alloc");
    WP_CUDA(ctx->d_Up.ensure(rtc), "alloc");
    WP_CUDA(ctx->d_allow.ensure((size_t)R * T), "alloc");
    WP_CUDA(ctx->d_Lpk.ensure(sizeof(uint32_t) * (size_t)R * T), "alloc");
    WP_CUDA(ctx->d_Upk.ensure(sizeof(uint32_t) * (size_t)R * T), "alloc");
    WP_CUDA(ctx->d_flags.ensure((size_t)R), "alloc");
    WP_CUDA(ctx->d_table.ensure(sizeof(EmitEntry) * (size_t)R * entries), "alloc emission table");
    // window-normalised factors for the engine (non-interacting models)
    const bool window_factors = !ctx->hm.interacting;
    if (window_factors) {
        WP_CUDA(ctx->d_gtab.ensure(sizeof(float) * (size_t)R * entries), "alloc window factors");
        WP_CUDA(ctx->d_gdelta.ensure((size_t)R * entries), "alloc window factors");
        WP_CUDA(ctx->d_gK.ensure(sizeof(int) * (size_t)R * T), "alloc window factors");
        WP_CUDA(ctx->d_gone.ensure(sizeof(float4) * (size_t)R * T), "alloc window factors");
    }
    WP_CUDA(ctx->d_err.ensure(sizeof(int)), "alloc");
    WP_CUDA(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(int), ctx->stream), "clear err");

    BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.model = ctx->d_model.as<DevModel>();
    a.peps = ctx->d_peps.as<PeptideRec>();
    a.counts = ctx->d_counts.as<int>();
    a.R = R;
    a.P = ctx->P;
    a.W = W;
    a.entries = entries;
    a.lo = ctx->d_lo.as<uint8_t>();
    a.hi = ctx->d_hi.as<uint8_t>();
    a.Lsuf = ctx->d_Ls.as<uint8_t>();
    a.Upre = ctx->d_Up.as<uint8_t>();
    a.allow = ctx->d_allow.as<uint8_t>();
    a.Lpk = ctx->d_Lpk.as<uint32_t>();
    a.Upk = ctx->d_Upk.as<uint32_t>();
    a.flags = ctx->d_flags.as<uint8_t>();
    a.tab = ctx->d_table.as<EmitEntry>();
    if (window_factors) {
        a.gtab = ctx->d_gtab.as<float>();
        a.gdelta = ctx->d_gdelta.as<uint8_t>();
        a.gK = ctx->d_gK.as<int>();
        a.gone = ctx->d_gone.as<float4>();
    }
    a.err = ctx->d_err.as<int>();

    {
        long n = (long)R * T;
        TimedLaunch tl(ctx, 1);
        wp_prep_reads_kernel<<<(int)((n + 127) / 128), 128, 0, ctx->stream>>>(
                a.model, d_rads, R, (unsigned)ctx->dmax, dist_cutoff, ctx->d_lo.as<uint8_t>(),
                ctx->d_hi.as<uint8_t>(), ctx->d_table.as<EmitEntry>(), entries);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "prep launch");
        wp_read_summary_kernel<<<(R + 127) / 128, 128, 0, ctx->stream>>>(a);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "summary launch");
        if (window_factors) {
            const size_t wsm = wp_window_smem_bytes(C, W, 128);
            WP_CUDA(cudaFuncSetAttribute(wp_window_factors_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)wsm), "window factors attribute");
            wp_window_factors_kernel<<<(int)((n + 127) / 128), 128, wsm, ctx->stream>>>(a);
            ctx->launches++;
            WP_CUDA(cudaGetLastError(), "window factors launch");
        }
    }
    if (mode == MODE_FLOPS) {
        long np = (long)R * ctx->P;
        TimedLaunch tl(ctx, 3);
        wp_count_flops_kernel<<<(int)((np + 127) / 128), 128, 0, ctx->stream>>>(a, d_flops);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "flops launch");
        return WP_OK;
    }
    if (d_cand_in) {
        a.cand = d_cand_in;
        a.slot_off = d_cand_off_in;
    } else if (h_cand) {
        WP_CUDA(ctx->d_cand.ensure(sizeof(int) * std::max<long>(n_slots, 1)), "alloc cand");
        WP_CUDA(ctx->d_slot_off.ensure(sizeof(int) * (R + 1)), "alloc cand");
        for (long k = 0; k < n_slots; k++)
            if (h_cand[k] < 0 || h_cand[k] >= ctx->P) return fail(ctx, WP_ERR_INVALID, "candidate index out of range");
        if (n_slots > 0)
            WP_CUDA(cudaMemcpyAsync(ctx->d_cand.p, h_cand, sizeof(int) * n_slots, cudaMemcpyHostToDevice, ctx->stream), "copy cand");
        WP_CUDA(cudaMemcpyAsync(ctx->d_slot_off.p, h_cand_off, sizeof(int) * (R + 1), cudaMemcpyHostToDevice, ctx->stream), "copy cand");
        a.cand = ctx->d_cand.as<int>();
        a.slot_off = ctx->d_slot_off.as<int>();
    } else {
        a.perm = ctx->d_perm.as<int>();
    }
    if (a.cand) a.shape_rank = ctx->d_shape_rank.as<int>();
    a.uniq_D = ctx->d_uniq_D.as<uint32_t>();
    a.pep_u = ctx->d_pep_u.as<int>();
    a.n_uniq = ctx->n_uniq_D;
    ctx->last_slots = n_slots;
    const size_t ns = (size_t)std::max<long>(n_slots, 1);
    WP_CUDA(ctx->d_res_mant.ensure(sizeof(float) * ns), "alloc results");
    WP_CUDA(ctx->d_res_expo.ensure(sizeof(int) * ns), "alloc results");
    // Classify over all peptides: the compaction works per group of
    // peptides with one dye-count vector and gives only non-empty pairs a
    // result index (BatchArgs::pair_info); loglik keeps one per slot.
    const bool groups = mode == MODE_CLASSIFY && !a.cand && ctx->n_grp <= WP_GROUP_MAX;
    if (groups) {
        a.grp_start = ctx->d_grp_start.as<int>();
        a.grp_D = ctx->d_grp_D.as<uint32_t>();
        a.n_grp = ctx->n_grp;
        WP_CUDA(ctx->d_pair_info.ensure(sizeof(int2) * ns), "alloc results");
        WP_CUDA(ctx->d_rd.ensure(sizeof(int) * 2 * (size_t)std::max(R, 1)), "alloc results");
        a.pair_info = ctx->d_pair_info.as<int2>();
        a.rd_base = ctx->d_rd.as<int>();
        a.rd_n = a.rd_base + R;
        // every read's range is written by the compaction; with no slots
        // the reduce reads none
    }
    WP_CUDA(ctx->d_work.ensure(sizeof(int2) * ns), "alloc work list");
    WP_CUDA(ctx->d_ovf1.ensure(sizeof(int2) * ns), "alloc work list");
    WP_CUDA(ctx->d_ovf2.ensure(sizeof(int2) * ns), "alloc work list");
    WP_CUDA(ctx->d_ovf3.ensure(sizeof(int2) * ns), "alloc work list");
    WP_CUDA(ctx->d_ovf4.ensure(sizeof(int2) * ns), "alloc work list");
    WP_CUDA(ctx->d_ovf5.ensure(sizeof(int2) * ns), "alloc work list");
    // counters (WP_CNT_*): list count / head per engine pass, the dense
    // kernel's, the non-empty pairs
    WP_CUDA(ctx->d_counters.ensure(sizeof(int) * WP_CNT_N), "alloc counters");
    WP_CUDA(cudaMemsetAsync(ctx->d_counters.p, 0, sizeof(int) * WP_CNT_N, ctx->stream), "clear counters");
    int* cnt = ctx->d_counters.as<int>();
    a.res_mant = ctx->d_res_mant.as<float>();
    a.res_expo = ctx->d_res_expo.as<int>();
    a.work = ctx->d_work.as<int2>();
    a.work_count = cnt + 0;
    a.work_head = cnt + 1;
    a.ovf = ctx->d_ovf2.as<int2>();
    a.ovf_count = cnt + WP_CNT_DENSE;
    a.ovf_head = cnt + WP_CNT_DENSE + 1;
    a.dense_S_cap = ((ctx->S_max + 31) / 32) * 32;
    if (n_slots > 0) {
        // Dense fallback shape: as many warps as fit (0: unavailable).
        int dense_warps = 0;
        for (int w = 16; w >= 1; w--)
            if (wp_dense_smem_bytes(T, a.dense_S_cap, C, hb, w) <= (size_t)ctx->smem_optin) {
                dense_warps = w;
                break;
            }
        // Pass 1 and pass 2 launch shapes (default: 2 CTAs of 256 threads
        // per SM, then 1 CTA of 256 with twice the slab); the dense kernel
        // takes what is left.
        const EngineCfg cfg = cfg_for(ctx);
        int half1 = slab_half_for(ctx, cfg.t1, cfg.s1, hb);
        int half2 = slab_half_for(ctx, cfg.t2, cfg.s2, hb);
        if (half1 < 4 || half2 < 4)
            return fail(ctx, WP_ERR_UNSUPPORTED, "shared memory too small for the pair engine");
        // Engine passes ("tiers") in order of growing slab: pass 1, a middle
        // pass of 3 CTAs of 128 threads per SM for the pairs just too large
        // for pass 1, the last configured pass, and passes of one CTA of 128
        // and of 64 threads per SM for what is left short of the dense
        // kernel (one thread per pair stays faster than the dense kernel's
        // warp over every state while the box fits).
        struct Tier {
            int threads, per_sm, half;
        };
        Tier tiers[WP_MAX_TIERS];
        int nt = 0;
        tiers[nt++] = {cfg.t1, cfg.s1, half1};
        const int hmid = slab_half_for(ctx, 128, 3, hb);
        if (hmid > half1 && hmid < half2) tiers[nt++] = {128, 3, hmid};
        if (half2 > tiers[nt - 1].half) tiers[nt++] = {cfg.t2, cfg.s2, half2};
        const int hbig = slab_half_for(ctx, 128, 1, hb);
        if (hbig > tiers[nt - 1].half) tiers[nt++] = {128, 1, hbig};
        const int hhuge = slab_half_for(ctx, 64, 1, hb);
        if (hhuge > tiers[nt - 1].half) tiers[nt++] = {64, 1, hhuge};
        DevBuf* lists[WP_MAX_TIERS] = {&ctx->d_work, &ctx->d_ovf1, &ctx->d_ovf3, &ctx->d_ovf4, &ctx->d_ovf5};
        // the compaction sends each pair to the first pass whose slab holds it
        a.n_tiers = nt;
        for (int k = 0; k < nt; k++) {
            a.tier_half[k] = tiers[k].half;
            a.tier_list[k] = lists[k]->as<int2>();
            a.tier_count[k] = cnt + 2 * k;
        }
        a.route_dense = dense_warps > 0 ? 1 : 0;
        a.live_count = cnt + WP_CNT_LIVE;
        {
            TimedLaunch tl(ctx, 1);
            if (groups) {
                // persistent: as many CTAs as are resident, at most one warp per read
                const size_t gsm = wp_compact_groups_smem_bytes(a.n_grp, a.P);
                WP_CUDA(cudaFuncSetAttribute(wp_compact_groups_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)gsm), "compact attribute");
                int per_sm = 0;
                WP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wp_compact_groups_kernel,
                                                                      WP_GROUP_WARPS * 32, gsm), "compact occupancy");
                int sms = 1;
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
                const int grid = std::max(1, std::min(sms * std::max(per_sm, 1),
                                                      (R + WP_GROUP_WARPS - 1) / WP_GROUP_WARPS));
                wp_compact_groups_kernel<<<grid, WP_GROUP_WARPS * 32, gsm, ctx->stream>>>(a);
            } else {
                wp_compact_kernel<<<R, 256, 0, ctx->stream>>>(a);
            }
            ctx->launches++;
            WP_CUDA(cudaGetLastError(), "compact launch");
        }
        for (int k = 0; k < nt; k++) {
            TimedLaunch tl(ctx, 0);
            const bool last = k + 1 == nt;
            size_t smem = wp_engine_smem_bytes(tiers[k].half, 0, hb, tiers[k].threads);
            WP_CUDA(wp_launch_engine(C, hb, tiers[k].threads, smem, ctx->stream, a, lists[k]->as<int2>(),
                                     cnt + 2 * k, cnt + 2 * k + 1,
                                     last ? ctx->d_ovf2.as<int2>() : lists[k + 1]->as<int2>(),
                                     last ? cnt + WP_CNT_DENSE : cnt + 2 * (k + 1), tiers[k].half, 0,
                                     last && dense_warps == 0 ? 1 : 0, k == 0 ? &ctx->last_engine_grid : nullptr),
                    "engine pass");
            ctx->launches++;
        }
        if (dense_warps > 0) {
            TimedLaunch tl(ctx, 0);
            size_t smem = wp_dense_smem_bytes(T, a.dense_S_cap, C, hb, dense_warps);
            WP_CUDA(wp_launch_dense(hb, dense_warps * 32, smem, ctx->stream, a), "dense launch");
            ctx->launches++;
        }
        if (mode == MODE_CLASSIFY) {
            EngineReplay& rp = ctx->replay;
            rp.a = a;
            rp.C = C;
            rp.T = T;
            rp.hb = hb;
            rp.nt = nt;
            rp.dense_warps = dense_warps;
            for (int k = 0; k < nt; k++) {
                rp.threads[k] = tiers[k].threads;
                rp.half[k] = tiers[k].half;
                rp.list[k] = lists[k]->as<int2>();
            }
            rp.cnt = cnt;
            rp.epoch = g_alloc_epoch;
            rp.valid = true;
        }
    }
    if (mode == MODE_CLASSIFY) {
        TimedLaunch tl(ctx, 2);
        wp_reduce_kernel<<<(R + 3) / 4, 128, 0, ctx->stream>>>(a, d_out_id, d_out_score, d_out_total,
                                                              d_out_log, ctx->d_ids.as<int>());
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "reduce launch");
    } else if (mode == MODE_LOGP && n_slots > 0) {
        TimedLaunch tl(ctx, 2);
        wp_logp_kernel<<<(int)((n_slots + 255) / 256), 256, 0, ctx->stream>>>(a.res_mant, a.res_expo,
                                                                              n_slots, d_logp);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "logp launch");
    }
    return WP_OK;
}

wp_status check_ready(wp_ctx* ctx) {
    if (!ctx->have_model) return fail(ctx, WP_ERR_STATE, "model not uploaded");
    if (!ctx->have_peps) return fail(ctx, WP_ERR_STATE, "peptides not uploaded");
    return WP_OK;
}

wp_status finish(wp_ctx* ctx) {
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    int err = 0;
    WP_CUDA(cudaMemcpy(&err, ctx->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (err == 2) return fail(ctx, WP_ERR_UNSUPPORTED, "a pair's state exceeds every shared-memory shape");
    if (err) return fail(ctx, WP_ERR_CUDA, "internal: peptide state exceeded its shape");
    return WP_OK;
}

// ChannelModel::adjusted_mu (parameterization/model/channel-model.h:35-54)
// on the host, for the kNN entry coordinates.
double host_adjusted_mu(const DevModel& m, int channel, const int* counts) {
    double amu = m.mu[channel] * (double)counts[channel];
    for (int c = 0; c < m.C; c++) {
        const double fi = m.flat[channel][c], ii = m.inter[channel][c];
        if (c == channel) {
            if (counts[c] > 1) {
                if (fi != 1.0) amu *= fi;
                if (ii != 1.0) amu *= std::pow(ii, (double)(counts[c] - 1));
            }
        } else if (counts[c] > 0) {
            if (fi != 1.0) amu *= fi;
            if (ii != 1.0) amu *= std::pow(ii, (double)counts[c]);
        }
    }
    return amu;
}

int nn_padded_dim(int TC) {
    for (int dp : {16, 32, 48, 64})
        if (TC <= dp) return dp;
    return -1;
}

// The kNN training set on the device for the current model and k: the
// entries in the order of the kd-tree NNClassifier builds over them
// (KDTree's constructor, kd-tree/kd-tree.h:36-43, with KDTEntry's
// coordinates, nn-classifier.cc:59-74), and with them their FP32
// coordinates, norms, hits and sources, the boxes of every 32 tree
// positions and of every leaf, the counts as bytes and the tree itself.
// Rebuilt when the model (coordinates) or k (leaf size) changes.
wp_status nn_prepare(wp_ctx* ctx, long long k) {
    const int T = ctx->nn_T, C = ctx->nn_C, N = ctx->nn_N, TC = T * C;
    const int DP = nn_padded_dim(TC);
    if (ctx->nn_coords_version == ctx->model_version && ctx->nn_tree_k == k) return WP_OK;
    // FP64 coordinates in input order
    std::vector<double> x64((size_t)std::max(N, 1) * TC, 0.0);
    int cts[WP_MAX_CHANNELS];
    int most = 0;
    bool bytes_ok = true;
    for (long e = 0; e < N; e++)
        for (int t = 0; t < T; t++) {
            for (int c = 0; c < C; c++) {
                cts[c] = ctx->nn_counts[(e * T + t) * C + c];
                if (cts[c] < 0 || cts[c] > 255) bytes_ok = false;
                most = std::max(most, cts[c]);
            }
            for (int c = 0; c < C; c++) x64[e * TC + t * C + c] = host_adjusted_mu(ctx->hm, c, cts);
        }
    const int kk = (int)std::min<long long>(k, INT32_MAX);
    if (wp_kdtree_build(x64.data(), N, TC, kk, &ctx->nn_perm, &ctx->nn_nodes, &ctx->nn_depth) != 0)
        return fail(ctx, WP_ERR_UNSUPPORTED, "kNN tree: shape not supported");
    const std::vector<int>& perm = ctx->nn_perm;
    // FP32 coordinates and squared norms in tree order
    std::vector<float> coords((size_t)std::max(N, 1) * DP, 0.0f);
    std::vector<float> norms(std::max(N, 1), 0.0f);
    for (long p = 0; p < N; p++) {
        const long e = perm[p];
        for (int i = 0; i < TC; i++) coords[p * DP + i] = (float)x64[e * TC + i];
        // squared norm in FP32, four partial sums as the kernels form |q|^2
        float q[4] = {0.f, 0.f, 0.f, 0.f};
        for (int i = 0; i < DP; i++) q[i % 4] = std::fma(coords[p * DP + i], coords[p * DP + i], q[i % 4]);
        norms[p] = (q[0] + q[1]) + (q[2] + q[3]);
    }
    // hits and sources in tree order
    std::vector<int> ehits(std::max(N, 1), 0), off(N + 1, 0);
    const int S = N > 0 ? ctx->nn_src_off[N] : 0;
    std::vector<int> dense(std::max(S, 1), 0), shits(std::max(S, 1), 0);
    std::vector<double> ratio(std::max(S, 1), 0.0);
    for (int p = 0; p < N; p++) {
        const int e = perm[p];
        int o = off[p];
        long long h = 0;
        for (int j = ctx->nn_src_off[e]; j < ctx->nn_src_off[e + 1]; j++, o++) {
            dense[o] = (int)(std::lower_bound(ctx->nn_uniq.begin(), ctx->nn_uniq.end(), ctx->nn_src_id[j]) -
                             ctx->nn_uniq.begin());
            ratio[o] = (double)ctx->nn_src_hits[j] / (double)ctx->nn_src_count[j];  // hits / count (nn-classifier.cc:154-158)
            shits[o] = ctx->nn_src_hits[j];
            h += ctx->nn_src_hits[j];
        }
        off[p + 1] = o;
        ehits[p] = (int)h;
    }
    // 16384 entries by systematic sampling of the cumulative hits (the
    // midpoint of each of 16384 equal shares): each stands for the same
    // number of hits, so the kNN search can estimate each read's k-hit
    // radius from them
    const int SN = N > 0 ? 16384 : 0;
    std::vector<int> sample(std::max(SN, 1), 0);
    {
        long long cum = 0;
        int p = 0;
        for (int j = 0; j < SN; j++) {
            const long long target = ((2ll * j + 1) * ctx->nn_hits_total) / (2ll * SN);
            while (p < N - 1 && cum + ehits[p] <= target) cum += ehits[p++];
            sample[j] = p;
        }
    }
    // per tile of 32 tree positions: bounding box of the coordinates and the
    // tile's hits (the kNN kernels skip tiles far from a read)
    const int nt = std::max((N + 31) / 32, 1);
    std::vector<float> tlo((size_t)nt * DP, 0.0f), thi((size_t)nt * DP, 0.0f);
    std::vector<int> ttot(nt, 0);
    for (int t = 0; t < (N + 31) / 32; t++) {
        const int e1 = std::min(N, 32 * t + 32);
        for (int i = 0; i < DP; i++) {
            float lo = coords[(size_t)32 * t * DP + i], hi = lo;
            for (int e = 32 * t + 1; e < e1; e++) {
                lo = std::min(lo, coords[(size_t)e * DP + i]);
                hi = std::max(hi, coords[(size_t)e * DP + i]);
            }
            tlo[(size_t)t * DP + i] = lo;
            thi[(size_t)t * DP + i] = hi;
        }
        long long h = 0;
        for (int e = 32 * t; e < e1; e++) h += ehits[e];
        ttot[t] = (int)std::min<long long>(h, INT32_MAX);
    }
    // per leaf: bounding box
    const int nn = std::max((int)ctx->nn_nodes.size(), 1);
    std::vector<float> llo((size_t)nn * DP, 0.0f), lhi((size_t)nn * DP, 0.0f);
    for (size_t id = 0; id < ctx->nn_nodes.size(); id++) {
        const KDNode& nd = ctx->nn_nodes[id];
        if (!nd.leaf) continue;
        for (int i = 0; i < DP; i++) {
            float lo = FLT_MAX, hi = -FLT_MAX;
            for (int p = nd.begin; p < nd.end; p++) {
                lo = std::min(lo, coords[(size_t)p * DP + i]);
                hi = std::max(hi, coords[(size_t)p * DP + i]);
            }
            llo[id * DP + i] = lo;
            lhi[id * DP + i] = hi;
        }
    }
    // counts as bytes and the coordinate of each count per channel
    // (non-interacting models), else FP64 coordinates, in tree order
    ctx->nn_inter = ctx->hm.interacting != 0;
    ctx->nn_NC = bytes_ok ? most + 1 : 0;
    std::vector<uint8_t> cnt8((size_t)std::max(N, 1) * DP, 0);
    if (bytes_ok)
        for (long p = 0; p < N; p++)
            for (int i = 0; i < TC; i++) cnt8[p * DP + i] = (uint8_t)ctx->nn_counts[(long)perm[p] * TC + i];
    std::vector<double> ctab((size_t)C * std::max(ctx->nn_NC, 1), 0.0);
    for (int c = 0; c < C; c++)
        for (int n = 0; n < ctx->nn_NC; n++) {
            int one[WP_MAX_CHANNELS] = {0, 0, 0, 0};
            one[c] = n;
            ctab[(size_t)c * ctx->nn_NC + n] = host_adjusted_mu(ctx->hm, c, one);
        }
    std::vector<double> ecoord;
    if (ctx->nn_inter) {
        ecoord.assign((size_t)std::max(N, 1) * TC, 0.0);
        for (long p = 0; p < N; p++)
            std::memcpy(&ecoord[p * TC], &x64[(size_t)perm[p] * TC], sizeof(double) * TC);
    }
    auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
        cudaError_t e = b.ensure(std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return e;
        return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    };
    WP_CUDA(up(ctx->d_nn_coords, coords.data(), sizeof(float) * coords.size()), "upload kNN coordinates");
    WP_CUDA(up(ctx->d_nn_enorm, norms.data(), sizeof(float) * norms.size()), "upload kNN norms");
    WP_CUDA(up(ctx->d_nn_hits, ehits.data(), sizeof(int) * ehits.size()), "upload kNN hits");
    WP_CUDA(up(ctx->d_nn_src_off, off.data(), sizeof(int) * off.size()), "upload kNN sources");
    WP_CUDA(up(ctx->d_nn_src_dense, dense.data(), sizeof(int) * dense.size()), "upload kNN sources");
    WP_CUDA(up(ctx->d_nn_src_ratio, ratio.data(), sizeof(double) * ratio.size()), "upload kNN sources");
    WP_CUDA(up(ctx->d_nn_src_hits, shits.data(), sizeof(int) * shits.size()), "upload kNN sources");
    WP_CUDA(up(ctx->d_nn_sample, sample.data(), sizeof(int) * sample.size()), "upload kNN sample");
    WP_CUDA(up(ctx->d_nn_tlo, tlo.data(), sizeof(float) * tlo.size()), "upload kNN tiles");
    WP_CUDA(up(ctx->d_nn_thi, thi.data(), sizeof(float) * thi.size()), "upload kNN tiles");
    WP_CUDA(up(ctx->d_nn_ttot, ttot.data(), sizeof(int) * ttot.size()), "upload kNN tiles");
    WP_CUDA(up(ctx->d_nn_llo, llo.data(), sizeof(float) * llo.size()), "upload kNN leaves");
    WP_CUDA(up(ctx->d_nn_lhi, lhi.data(), sizeof(float) * lhi.size()), "upload kNN leaves");
    WP_CUDA(up(ctx->d_nn_cnt8, cnt8.data(), cnt8.size()), "upload kNN counts");
    WP_CUDA(up(ctx->d_nn_ctab, ctab.data(), sizeof(double) * ctab.size()), "upload kNN count table");
    if (ctx->nn_inter) WP_CUDA(up(ctx->d_nn_ecoord, ecoord.data(), sizeof(double) * ecoord.size()), "upload kNN coordinates");
    if (!ctx->nn_nodes.empty())
        WP_CUDA(up(ctx->d_nn_nodes, ctx->nn_nodes.data(), sizeof(KDNode) * ctx->nn_nodes.size()), "upload kNN tree");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->nn_sample_n = SN;
    ctx->nn_coords_version = ctx->model_version;
    ctx->nn_tree_k = k;
    return WP_OK;
}

// Peptide index and count of each source id for the hybrid classifier
// (hybrid-classifier.cc:46-50); ids absent from the peptide set read as
// index 0 and count 0, as the reference's unordered_map operator[] gives.
wp_status nn_prepare_peptides(wp_ctx* ctx) {
    if (ctx->nn_pep_version == ctx->pep_version) return WP_OK;
    std::vector<std::pair<int, int>> idx;
    idx.reserve(ctx->P);
    for (int i = 0; i < ctx->P; i++) idx.push_back({ctx->ids[i], i});
    std::sort(idx.begin(), idx.end());
    std::vector<int> pep(std::max(ctx->nn_U, 1), 0), cnt(std::max(ctx->nn_U, 1), 0);
    for (int u = 0; u < ctx->nn_U; u++) {
        const int id = ctx->nn_uniq[u];
        auto it = std::lower_bound(idx.begin(), idx.end(), std::make_pair(id, INT32_MIN));
        // the map keeps the last peptide with a repeated id
        int found = -1;
        while (it != idx.end() && it->first == id) found = (it++)->second;
        if (found >= 0) {
            pep[u] = found;
            cnt[u] = ctx->counts[found];
        }
    }
    WP_CUDA(ctx->d_nn_dense_pep.ensure(sizeof(int) * pep.size()), "alloc");
    WP_CUDA(ctx->d_nn_dense_count.ensure(sizeof(int) * cnt.size()), "alloc");
    WP_CUDA(cudaMemcpyAsync(ctx->d_nn_dense_pep.p, pep.data(), sizeof(int) * pep.size(), cudaMemcpyHostToDevice,
                            ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(ctx->d_nn_dense_count.p, cnt.data(), sizeof(int) * cnt.size(), cudaMemcpyHostToDevice,
                            ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->nn_pep_version = ctx->pep_version;
    return WP_OK;
}

// The reference's k-hit set for R query slots (wp_kbest.cu): per slot the
// final top of KBest.  Slots whose scratch ran out are replayed again by
// fewer warps with four times the scratch, then sixteen times.
wp_status nn_replay(wp_ctx* ctx, const double* d_rads, int R, long long k) {
    const int T = ctx->nn_T, C = ctx->nn_C, TC = T * C;
    if (ctx->nn_NC == 0) return fail(ctx, WP_ERR_UNSUPPORTED, "kd-tree kNN needs dye counts in 0..255");
    const size_t Rz = (size_t)std::max(R, 1);
    WP_CUDA(ctx->d_kb_tfd.ensure(sizeof(double) * Rz), "alloc");
    WP_CUDA(ctx->d_kb_tfpos.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_kb_tfflag.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_kb_next.ensure(sizeof(int)), "alloc");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    KBArgs a;
    memset(&a, 0, sizeof(a));
    a.next = ctx->d_kb_next.as<int>();
    a.qperm = ctx->d_nn_qperm.as<int>();
    a.rads = d_rads;
    a.TC = TC;
    a.C = C;
    a.DP = nn_padded_dim(TC);
    a.N = ctx->nn_N;
    a.k = k;
    a.cnt = ctx->d_nn_cnt8.as<uint8_t>();
    a.ctab = ctx->d_nn_ctab.as<double>();
    a.NC = ctx->nn_NC;
    a.interact = ctx->nn_inter ? 1 : 0;
    a.ecoord = ctx->nn_inter ? ctx->d_nn_ecoord.as<double>() : nullptr;
    a.coords32 = ctx->d_nn_coords.as<float>();
    a.tlo = ctx->d_nn_tlo.as<float>();
    a.thi = ctx->d_nn_thi.as<float>();
    a.llo = ctx->d_nn_llo.as<float>();
    a.lhi = ctx->d_nn_lhi.as<float>();
    a.hits = ctx->d_nn_hits.as<int>();
    a.nodes = ctx->d_nn_nodes.as<KDNode>();
    a.stack_cap = ctx->nn_depth + 2;
    a.tf_d = ctx->d_kb_tfd.as<double>();
    a.tf_pos = ctx->d_kb_tfpos.as<int>();
    a.tf_flag = ctx->d_kb_tfflag.as<int>();
    const size_t smem = wp_kbest_smem_bytes(TC, a.NC, a.stack_cap, a.interact != 0);
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if (smem > (size_t)dev_smem) return fail(ctx, WP_ERR_UNSUPPORTED, "kd-tree kNN: per-read tables exceed shared memory");
    // as many CTAs per SM as its shared memory holds (each warp walks one read
    // at a time, latency-bound: residency is what speeds it up)
    const int per_sm = std::max(1, std::min(8, (int)((size_t)(228 * 1024) / (smem + 1024))));
    const int ch = wp_kbest_chunk();
    std::vector<int> redo;
    for (int round = 0; round < 3; round++) {
        // live entries stay below about k plus the extras KBest keeps
        const long long grow = 1ll << (2 * round);
        const long long stage = std::min<long long>((std::max<long long>(32768, 2 * k + 8192)) * grow, 1ll << 26);
        a.stagecap = (int)stage;
        a.regcap = (int)(((2 * stage + 2048ll * ch) + ch - 1) / ch * ch);
        if (a.regcap / ch > 65535) a.regcap = 65535 * ch;
        int grid = sms * per_sm;
        if (round > 0) {
            const int wpc = wp_kbest_warps_per_cta();
            grid = std::max(1, std::min(grid, ((int)redo.size() + wpc - 1) / wpc));
        }
        const long warps = (long)grid * wp_kbest_warps_per_cta();
        WP_CUDA(ctx->d_kb_reg.ensure(sizeof(KBItem) * 2 * (size_t)a.regcap * warps), "alloc kNN replay scratch");
        WP_CUDA(ctx->d_kb_prev.ensure(sizeof(int) * 2 * (size_t)(a.regcap / ch) * warps), "alloc kNN replay scratch");
        WP_CUDA(ctx->d_kb_stage.ensure(sizeof(KBItem) * (size_t)a.stagecap * warps), "alloc kNN replay scratch");
        a.reg = ctx->d_kb_reg.as<KBItem>();
        a.prev = ctx->d_kb_prev.as<int>();
        a.stage = ctx->d_kb_stage.as<KBItem>();
        if (round == 0) {
            a.nwork = R;
            a.work = nullptr;
        } else {
            WP_CUDA(ctx->d_kb_work.ensure(sizeof(int) * redo.size()), "alloc");
            WP_CUDA(cudaMemcpyAsync(ctx->d_kb_work.p, redo.data(), sizeof(int) * redo.size(), cudaMemcpyHostToDevice,
                                    ctx->stream), "copy");
            a.nwork = (int)redo.size();
            a.work = ctx->d_kb_work.as<int>();
        }
        WP_CUDA(cudaMemsetAsync(a.next, 0, sizeof(int), ctx->stream), "clear");
        {
            TimedLaunch tl(ctx, 8);
            WP_CUDA(wp_launch_kbest(grid, ctx->stream, a), "kNN kd-tree replay");
            ctx->launches++;
        }
        std::vector<int> flags(R);
        WP_CUDA(cudaMemcpyAsync(flags.data(), a.tf_flag, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        redo.clear();
        for (int r = 0; r < R; r++)
            if (flags[r] & 4) redo.push_back(r);
        if (redo.empty()) return WP_OK;
    }
    return fail(ctx, WP_ERR_UNSUPPORTED, "kd-tree kNN: replay scratch exhausted");
}

// The kNN stage for R reads already on the device (FP64 [R][T][C]):
// per read the top-h candidates in ascending (score, id) order, the total
// and, when hybrid, candidate peptide indices and the subfraction.
wp_status nn_run(wp_ctx* ctx, const double* d_rads, int R, int k, double sig, int h, bool hybrid) {
    const int T = ctx->nn_T, C = ctx->nn_C, N = ctx->nn_N;
    const int DP = nn_padded_dim(T * C);
    wp_status st = nn_prepare(ctx, k);
    if (st != WP_OK) return st;
    const bool exact = ctx->nn_selection == WP_NN_KDTREE;
    if (hybrid) {
        st = nn_prepare_peptides(ctx);
        if (st != WP_OK) return st;
    }
    const size_t Rz = (size_t)std::max(R, 1);
    WP_CUDA(ctx->d_nn_queries.ensure(sizeof(float) * Rz * DP), "alloc queries");
    WP_CUDA(ctx->d_nn_qbin.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_qbase.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_qbelow.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_qcap.ensure(sizeof(long long) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_qoff.ensure(sizeof(long long) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_ncand.ensure(sizeof(int) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_cand_id.ensure(sizeof(int) * Rz * h), "alloc");
    WP_CUDA(ctx->d_nn_cand_pep.ensure(sizeof(int) * Rz * h), "alloc");
    WP_CUDA(ctx->d_nn_cand_score.ensure(sizeof(double) * Rz * h), "alloc");
    WP_CUDA(ctx->d_nn_total.ensure(sizeof(double) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_subfrac.ensure(sizeof(double) * Rz), "alloc");
    WP_CUDA(ctx->d_nn_err.ensure(sizeof(int)), "alloc");
    WP_CUDA(cudaMemsetAsync(ctx->d_nn_err.p, 0, sizeof(int), ctx->stream), "clear");
    if (R == 0) return WP_OK;
    if (N == 0) {
        WP_CUDA(cudaMemsetAsync(ctx->d_nn_ncand.p, 0, sizeof(int) * R, ctx->stream), "clear");
        WP_CUDA(cudaMemsetAsync(ctx->d_nn_total.p, 0, sizeof(double) * R, ctx->stream), "clear");
        WP_CUDA(cudaMemsetAsync(ctx->d_nn_subfrac.p, 0, sizeof(double) * R, ctx->stream), "clear");
        return WP_OK;
    }
    WP_CUDA(wp_launch_nn_queries(d_rads, R, T * C, DP, ctx->d_nn_queries.as<float>(), ctx->stream), "queries");
    ctx->launches++;
    // reads in an order that groups alike ones (results go back by perm)
    {
        WP_CUDA(ctx->d_nn_qsorted.ensure(sizeof(float) * Rz * DP), "alloc");
        WP_CUDA(ctx->d_nn_qperm.ensure(sizeof(int) * Rz), "alloc");
        WP_CUDA(ctx->d_nn_qkeys.ensure(sizeof(unsigned long long) * 2 * Rz), "alloc");
        WP_CUDA(ctx->d_nn_qidx.ensure(sizeof(int) * 2 * Rz), "alloc");
        const size_t tb = wp_nn_sort_temp_bytes(R);
        WP_CUDA(ctx->d_nn_qtemp.ensure(std::max<size_t>(tb, 1)), "alloc");
        WP_CUDA(wp_launch_nn_sort_queries(ctx->d_nn_queries.as<float>(), R, DP, T * C, ctx->d_nn_qsorted.as<float>(),
                                          ctx->d_nn_qperm.as<int>(), ctx->d_nn_qkeys.as<unsigned long long>(),
                                          ctx->d_nn_qidx.as<int>(), ctx->d_nn_qtemp.p, tb, ctx->stream),
                "sort queries");
        ctx->launches += 3;
    }
    if (exact) {
        st = nn_replay(ctx, d_rads, R, k);
        if (st != WP_OK) return st;
    }
    NNArgs a;
    memset(&a, 0, sizeof(a));
    a.coords = ctx->d_nn_coords.as<float>();
    a.enorm = ctx->d_nn_enorm.as<float>();
    a.tlo = ctx->d_nn_tlo.as<float>();
    a.thi = ctx->d_nn_thi.as<float>();
    a.ttot = ctx->d_nn_ttot.as<int>();
    a.hits = ctx->d_nn_hits.as<int>();
    a.N = N;
    a.k = k;
    a.qbin = ctx->d_nn_qbin.as<int>();
    a.qbelow = ctx->d_nn_qbelow.as<int>();
    a.qcap = ctx->d_nn_qcap.as<long long>();
    a.err = ctx->d_nn_err.as<int>();
    a.qbase = ctx->d_nn_qbase.as<int>();
    a.sample = ctx->d_nn_sample.as<int>();
    a.sample_n = ctx->nn_sample_n;
    a.hits_total = ctx->nn_hits_total;
    a.tf_d = exact ? ctx->d_kb_tfd.as<double>() : nullptr;
    a.tf_flag = exact ? ctx->d_kb_tfflag.as<int>() : nullptr;
    // Entry slices: enough CTAs (query blocks x slices) for two waves of
    // three CTAs per SM, each slice at least 1024 entries.
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    {
        const int qblocks = (R + wp_nn_queries_per_block() - 1) / wp_nn_queries_per_block();
        int slices = (6 * sms + qblocks - 1) / qblocks;
        slices = std::max(1, std::min(slices, std::min(32, (N + 1023) / 1024)));
        a.slices = slices;
        a.slice_len = ((N + slices - 1) / slices + 31) / 32 * 32;
        a.slices = (N + a.slice_len - 1) / a.slice_len;
    }
    a.R_all = R;
    WP_CUDA(ctx->d_nn_shist.ensure(sizeof(unsigned) * (size_t)a.slices * R * wp_nn_bins()), "alloc kNN histograms");
    WP_CUDA(ctx->d_nn_sliceoff.ensure(sizeof(long long) * (size_t)a.slices * R), "alloc");
    WP_CUDA(ctx->d_nn_slicecap.ensure(sizeof(long long) * (size_t)a.slices * R), "alloc");
    WP_CUDA(ctx->d_nn_slicecnt.ensure(sizeof(long long) * (size_t)a.slices * R), "alloc");
    a.shist = ctx->d_nn_shist.as<unsigned>();
    a.n_super = a.slices * ((a.slice_len + 1023) / 1024);
    WP_CUDA(ctx->d_nn_stmin.ensure((size_t)R * a.n_super), "alloc kNN super-tile bins");
    a.stmin = ctx->d_nn_stmin.as<unsigned char>();
    a.sliceoff = ctx->d_nn_sliceoff.as<long long>();
    a.slicecap = ctx->d_nn_slicecap.as<long long>();
    a.slicecnt = ctx->d_nn_slicecnt.as<long long>();
    // pass 1 over every read: the bins' origins from a sample, then the
    // histograms
    a.queries = ctx->d_nn_qsorted.as<float>();
    a.R = R;
    a.q0 = 0;
    {
        TimedLaunch tl(ctx, 4);
        WP_CUDA(wp_launch_nn_estimate(DP, ctx->stream, a), "kNN estimate");
        ctx->launches++;
    }
    {
        TimedLaunch tl(ctx, 4);
        WP_CUDA(wp_launch_nn_dist(DP, true, ctx->stream, a), "kNN histogram");
        ctx->launches++;
    }
    WP_CUDA(wp_launch_nn_threshold(ctx->stream, a), "kNN threshold");
    ctx->launches++;
    // reads whose k-th hit lies beyond their bins: counted again with the
    // bins moved up 2.5 octaves (at most three times; after that the open
    // last bin is just a large candidate set)
    WP_CUDA(ctx->d_nn_redo.ensure(sizeof(int) * (Rz + 1)), "alloc");
    for (int round = 0; round < 3; round++) {
        int* list = ctx->d_nn_redo.as<int>() + 1;
        WP_CUDA(wp_launch_nn_redo(a, list, ctx->d_nn_redo.as<int>(), 40, ctx->stream), "kNN redo");
        ctx->launches++;
        int nredo = 0;
        WP_CUDA(cudaMemcpyAsync(&nredo, ctx->d_nn_redo.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        if (nredo == 0) break;
        NNArgs r = a;
        r.slots = list;
        r.R = nredo;
        // few reads: each entry slice split over enough CTAs to fill the
        // device, their counts added into the (zeroed) slice histograms
        const int qb = (nredo + wp_nn_queries_per_block() - 1) / wp_nn_queries_per_block();
        r.sub = std::max(1, std::min(64, (3 * sms) / std::max(1, qb * a.slices)));
        if (r.sub > 1) {
            WP_CUDA(wp_launch_nn_zero_hist(r, ctx->stream), "kNN zero");
            ctx->launches++;
        }
        {
            TimedLaunch tl(ctx, 4);
            WP_CUDA(wp_launch_nn_dist(DP, true, ctx->stream, r), "kNN histogram");
            ctx->launches++;
        }
        r.sub = 0;
        WP_CUDA(wp_launch_nn_threshold(ctx->stream, r), "kNN threshold");
        ctx->launches++;
    }
    std::vector<long long> cap(R);
    WP_CUDA(cudaMemcpyAsync(cap.data(), a.qcap, sizeof(long long) * R, cudaMemcpyDeviceToHost, ctx->stream),
            "copy caps");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    // per-warp accumulators of the select kernel
    const int sel_grid = sms * 4;
    const long nwarps = (long)sel_grid * wp_nn_select_warps();
    const int U = std::max(ctx->nn_U, 1);
    WP_CUDA(ctx->d_nn_acc.ensure(sizeof(double) * nwarps * U), "alloc kNN accumulators");
    WP_CUDA(ctx->d_nn_mark.ensure(sizeof(int) * nwarps * U), "alloc kNN accumulators");
    WP_CUDA(ctx->d_nn_touched.ensure(sizeof(int) * nwarps * U), "alloc kNN accumulators");
    // The select kernel leaves every accumulator it touched at zero again,
    // so memory is cleared once, when first used.
    if (sizeof(double) * nwarps * U > ctx->nn_acc_cleared) {
        WP_CUDA(cudaMemsetAsync(ctx->d_nn_acc.p, 0, sizeof(double) * nwarps * U, ctx->stream), "clear");
        WP_CUDA(cudaMemsetAsync(ctx->d_nn_mark.p, 0, sizeof(int) * nwarps * U, ctx->stream), "clear");
        ctx->nn_acc_cleared = sizeof(double) * nwarps * U;
    }
    // chunks of reads whose candidate lists fit the budget
    const long long budget = 256ll << 20;  // candidates per chunk (2 GiB of lists)
    int r0 = 0;
    std::vector<long long> off;
    while (r0 < R) {
        long long tot = 0;
        int r1 = r0;
        off.clear();
        while (r1 < R && (r1 == r0 || tot + cap[r1] <= budget)) {
            off.push_back(tot);
            tot += cap[r1];
            r1++;
        }
        const int nq = r1 - r0;
        WP_CUDA(ctx->d_nn_cidx.ensure(sizeof(int) * std::max<long long>(tot, 1)), "alloc kNN candidates");
        WP_CUDA(ctx->d_nn_cd2.ensure(sizeof(float) * std::max<long long>(tot, 1)), "alloc kNN candidates");
        WP_CUDA(ctx->d_nn_chits.ensure(sizeof(int) * std::max<long long>(tot, 1)), "alloc kNN candidates");
        WP_CUDA(ctx->d_nn_cbin.ensure(std::max<long long>(tot, 1)), "alloc kNN candidates");
        WP_CUDA(cudaMemcpyAsync(ctx->d_nn_qoff.p, off.data(), sizeof(long long) * nq, cudaMemcpyHostToDevice,
                                ctx->stream), "copy offsets");
        a.queries = ctx->d_nn_qsorted.as<float>() + (size_t)r0 * DP;
        a.R = nq;
        a.q0 = r0;
        a.qoff = ctx->d_nn_qoff.as<long long>();
        a.cand_idx = ctx->d_nn_cidx.as<int>();
        a.cand_d2 = ctx->d_nn_cd2.as<float>();
        a.cand_hits = ctx->d_nn_chits.as<int>();
        a.cand_bin = ctx->d_nn_cbin.as<unsigned char>();
        {
            TimedLaunch tl(ctx, 4);
            WP_CUDA(wp_launch_nn_dist(DP, false, ctx->stream, a), "kNN collect");
            ctx->launches++;
        }
        NNSelectArgs b;
        memset(&b, 0, sizeof(b));
        b.R = nq;
        b.q0 = r0;
        b.qbin = a.qbin;
        b.qperm = ctx->d_nn_qperm.as<int>();
        b.qbase = a.qbase;
        b.qbelow = a.qbelow;
        b.slices = a.slices;
        b.R_all = R;
        b.sliceoff = a.sliceoff;
        b.slicecnt = a.slicecnt;
        b.slicecap = a.slicecap;
        b.qoff = a.qoff;
        b.cand_idx = a.cand_idx;
        b.cand_d2 = a.cand_d2;
        b.cand_hits = a.cand_hits;
        b.cand_bin = a.cand_bin;
        b.hits = a.hits;
        b.src_off = ctx->d_nn_src_off.as<int>();
        b.src_dense = ctx->d_nn_src_dense.as<int>();
        b.src_ratio = ctx->d_nn_src_ratio.as<double>();
        b.src_hits = ctx->d_nn_src_hits.as<int>();
        b.dense_id = ctx->d_nn_dense_id.as<int>();
        b.dense_pep = hybrid ? ctx->d_nn_dense_pep.as<int>() : nullptr;
        b.dense_count = hybrid ? ctx->d_nn_dense_count.as<int>() : nullptr;
        b.U = U;
        b.k = k;
        b.inv_two_sig_sq = (float)(1.0 / (2.0 * sig * sig));
        b.h = h;
        b.acc = ctx->d_nn_acc.as<double>();
        b.mark = ctx->d_nn_mark.as<int>();
        b.touched = ctx->d_nn_touched.as<int>();
        b.out_ncand = ctx->d_nn_ncand.as<int>();
        b.out_cand_id = ctx->d_nn_cand_id.as<int>();
        b.out_cand_pep = hybrid ? ctx->d_nn_cand_pep.as<int>() : nullptr;
        b.out_cand_score = ctx->d_nn_cand_score.as<double>();
        b.out_total = ctx->d_nn_total.as<double>();
        b.out_subfrac = hybrid ? ctx->d_nn_subfrac.as<double>() : nullptr;
        b.two_sig_sq = 2.0 * sig * sig;
        if (ctx->nn_NC > 0) {
            b.rads = d_rads;
            b.TC = T * C;
            b.C = C;
            b.DP = DP;
            b.NC = ctx->nn_NC;
            b.cnt = ctx->d_nn_cnt8.as<uint8_t>();
            b.ctab = ctx->d_nn_ctab.as<double>();
            b.ecoord = ctx->nn_inter ? ctx->d_nn_ecoord.as<double>() : nullptr;
        }
        if (exact) {
            b.tf_d = ctx->d_kb_tfd.as<double>();
            b.tf_pos = ctx->d_kb_tfpos.as<int>();
            b.tf_flag = ctx->d_kb_tfflag.as<int>();
            b.rads = d_rads;
            b.TC = T * C;
            b.C = C;
            b.DP = DP;
            b.NC = ctx->nn_NC;
            b.cnt = ctx->d_nn_cnt8.as<uint8_t>();
            b.ctab = ctx->d_nn_ctab.as<double>();
            b.ecoord = ctx->nn_inter ? ctx->d_nn_ecoord.as<double>() : nullptr;
        }
        {
            TimedLaunch tl(ctx, 5);
            WP_CUDA(wp_launch_nn_select(sel_grid, ctx->stream, b), "kNN select");
            ctx->launches++;
        }
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        r0 = r1;
    }
    int err = 0;
    WP_CUDA(cudaMemcpy(&err, ctx->d_nn_err.p, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (err) return fail(ctx, WP_ERR_CUDA, "internal: kNN candidate list overflow");
    return WP_OK;
}

wp_status nn_check(wp_ctx* ctx, int k, double sig, int h) {
    if (!ctx->have_model) return fail(ctx, WP_ERR_STATE, "model not uploaded");
    if (!ctx->have_tracks) return fail(ctx, WP_ERR_STATE, "dye-tracks not uploaded");
    if (ctx->nn_T != ctx->hm.T || ctx->nn_C != ctx->hm.C)
        return fail(ctx, WP_ERR_STATE, "dye-track shape differs from the model's timesteps/channels");
    if (k < 1) return fail(ctx, WP_ERR_INVALID, "k must be >= 1");
    if (!(sig > 0.0)) return fail(ctx, WP_ERR_INVALID, "sig must be > 0");
    if (h < 1 || h > wp_nn_hmax()) return fail(ctx, WP_ERR_UNSUPPORTED, "h must be in 1..1024");
    return WP_OK;
}

wp_status hybrid_check(wp_ctx* ctx, int k, double sig, int h) {
    wp_status st = nn_check(ctx, k, sig, h);
    if (st != WP_OK) return st;
    st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (ctx->P == 0) return fail(ctx, WP_ERR_INVALID, "the hybrid classifier needs at least one peptide");
    return WP_OK;
}

// HybridClassifier::classify (hybrid-classifier.cc:55-81) for reads on the
// device: kNN candidates, the HMM over them (ascending kNN score), then the
// score scaled by the candidates' subfraction and NaN patched on the device.
wp_status hybrid_run(wp_ctx* ctx, const double* d_rads, int R, int k, double sig, int h, double dist_cutoff,
                     int* d_out_id, double* d_out_score, double* d_out_total) {
    wp_status st = nn_run(ctx, d_rads, R, k, sig, h, true);
    if (st != WP_OK) return st;
    std::vector<int> ncand(R), off(R + 1, 0);
    WP_CUDA(cudaMemcpyAsync(ncand.data(), ctx->d_nn_ncand.p, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    for (int r = 0; r < R; r++) off[r + 1] = off[r] + ncand[r];
    WP_CUDA(ctx->d_nn_cand_off.ensure(sizeof(int) * (R + 1)), "alloc");
    WP_CUDA(ctx->d_nn_cand_flat.ensure(sizeof(int) * std::max(off[R], 1)), "alloc");
    WP_CUDA(cudaMemcpyAsync(ctx->d_nn_cand_off.p, off.data(), sizeof(int) * (R + 1), cudaMemcpyHostToDevice, ctx->stream), "copy");
    WP_CUDA(wp_launch_nn_ragged(ctx->d_nn_cand_pep.as<int>(), h, ctx->d_nn_cand_off.as<int>(), R,
                                ctx->d_nn_cand_flat.as<int>(), ctx->stream), "ragged");
    ctx->launches++;
    st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, off.data(), MODE_CLASSIFY, nullptr, d_out_id, d_out_score,
                   d_out_total, nullptr, nullptr, ctx->d_nn_cand_flat.as<int>(), ctx->d_nn_cand_off.as<int>());
    if (st != WP_OK) return st;
    WP_CUDA(wp_launch_hybrid_finish(ctx->d_nn_ncand.as<int>(), ctx->d_nn_subfrac.as<double>(), R, d_out_id,
                                    d_out_score, d_out_total, ctx->stream), "hybrid finish");
    ctx->launches++;
    return WP_OK;
}

// Reads simulated on the device from the context's model and peptides.
wp_status sim_device(wp_ctx* ctx, int R, unsigned long long seed, float* d_rads_f, double* d_rads_d, int* d_pep,
                     uint8_t* d_tracks, int per_peptide = 0) {
    if (ctx->sim_pep_version != ctx->pep_version) {
        std::vector<int8_t> seqs(std::max<size_t>(ctx->seqs.size(), 1), -1);
        for (size_t i = 0; i < ctx->seqs.size(); i++) seqs[i] = (int8_t)ctx->seqs[i];
        std::vector<double> cum(std::max(ctx->P, 1), 0.0);
        double acc = 0.0;
        for (int i = 0; i < ctx->P; i++) {
            acc += (double)ctx->counts[i];
            cum[i] = acc;
        }
        if (ctx->P > 0 && !(acc > 0.0)) return fail(ctx, WP_ERR_INVALID, "peptide counts sum to zero");
        int most = 0;
        for (int i = 0; i < ctx->P; i++) {
            int per[WP_MAX_CHANNELS] = {0, 0, 0, 0};
            for (int j = ctx->offsets[i]; j < ctx->offsets[i + 1]; j++)
                if (ctx->seqs[j] >= 0 && ctx->seqs[j] < WP_MAX_CHANNELS) most = std::max(most, ++per[ctx->seqs[j]]);
        }
        ctx->sim_max_dyes = most;
        WP_CUDA(ctx->d_sim_ids.ensure(sizeof(int) * std::max(ctx->P, 1)), "alloc");
        WP_CUDA(ctx->d_sim_cnts.ensure(sizeof(int) * std::max(ctx->P, 1)), "alloc");
        WP_CUDA(cudaMemcpyAsync(ctx->d_sim_ids.p, ctx->ids.data(), sizeof(int) * ctx->P, cudaMemcpyHostToDevice,
                                ctx->stream), "copy");
        WP_CUDA(cudaMemcpyAsync(ctx->d_sim_cnts.p, ctx->counts.data(), sizeof(int) * ctx->P, cudaMemcpyHostToDevice,
                                ctx->stream), "copy");
        WP_CUDA(ctx->d_sim_seqs.ensure(seqs.size()), "alloc");
        WP_CUDA(ctx->d_sim_off.ensure(sizeof(int) * ctx->offsets.size()), "alloc");
        WP_CUDA(ctx->d_sim_cum.ensure(sizeof(double) * cum.size()), "alloc");
        WP_CUDA(cudaMemcpyAsync(ctx->d_sim_seqs.p, seqs.data(), seqs.size(), cudaMemcpyHostToDevice, ctx->stream), "copy");
        WP_CUDA(cudaMemcpyAsync(ctx->d_sim_off.p, ctx->offsets.data(), sizeof(int) * ctx->offsets.size(),
                                cudaMemcpyHostToDevice, ctx->stream), "copy");
        WP_CUDA(cudaMemcpyAsync(ctx->d_sim_cum.p, cum.data(), sizeof(double) * cum.size(), cudaMemcpyHostToDevice,
                                ctx->stream), "copy");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        ctx->sim_pep_version = ctx->pep_version;
    }
    SimParams p;
    memset(&p, 0, sizeof(p));
    p.T = ctx->hm.T;
    p.C = ctx->hm.C;
    p.P = ctx->P;
    p.R = R;
    p.seed = seed;
    // ceil(p * 2^32) (exact in FP64), 0 for p <= 0, 2^32 for p >= 1
    auto thr = [](double q) -> unsigned long long {
        if (!(q > 0.0)) return 0ull;
        if (q >= 1.0) return 1ull << 32;
        return (unsigned long long)ceil(q * 4294967296.0);
    };
    p.thr_fail = thr(ctx->raw_pf);
    p.thr_initial_block = thr(ctx->raw_pib);
    p.thr_cyclic_block = thr(ctx->raw_pcb);
    for (int t = 0; t < WP_MAX_TIMESTEPS; t++) p.thr_detach[t] = thr(ctx->raw_pdet[t]);
    for (int c = 0; c < WP_MAX_CHANNELS; c++) {
        p.thr_dud[c] = thr(ctx->raw_pdud[c]);
        p.thr_bleach[c] = thr(ctx->raw_pbleach[c]);
    }
    p.model = ctx->d_model.as<DevModel>();
    p.seqs = ctx->d_sim_seqs.as<int8_t>();
    p.offsets = ctx->d_sim_off.as<int>();
    p.cum = ctx->d_sim_cum.as<double>();
    p.rads_f = d_rads_f;
    p.rads_d = d_rads_d;
    p.pep = d_pep;
    p.tracks = d_tracks;
    p.per_peptide = per_peptide;
    TimedLaunch tl(ctx, 6);
    WP_CUDA(wp_launch_sim_reads(p, ctx->stream), "simulator launch");
    ctx->launches++;
    return WP_OK;
}

wp_status upload_reads(wp_ctx* ctx, const double* rads, int R) {
    const size_t bytes = sizeof(double) * (size_t)R * ctx->hm.T * ctx->hm.C;
    WP_CUDA(ctx->d_rads.ensure(bytes), "alloc reads");
    WP_CUDA(cudaMemcpyAsync(ctx->d_rads.p, rads, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy reads");
    return WP_OK;
}

}  // namespace

extern "C" {

wp_status wp_ctx_create(wp_ctx** out, int device) {
    if (!out) return WP_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || device < 0 || device >= n) return WP_ERR_CUDA;
    wp_ctx* ctx = new (std::nothrow) wp_ctx();
    if (!ctx) return WP_ERR_OOM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return WP_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (ctx->d_model.ensure(sizeof(DevModel)) != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return WP_ERR_OOM;
    }
    *out = ctx;
    return WP_OK;
}

void wp_ctx_destroy(wp_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    collect_timing(ctx);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* wp_last_error(const wp_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long wp_launch_count(const wp_ctx* ctx) { return ctx ? ctx->launches : 0; }

void* wp_ctx_stream(const wp_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

wp_status wp_last_batch_stats(wp_ctx* ctx, long long* stats) {
    if (!ctx || !stats) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int c[WP_CNT_N] = {0};
    if (ctx->d_counters.p) {
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        WP_CUDA(cudaMemcpy(c, ctx->d_counters.p, sizeof(c), cudaMemcpyDeviceToHost), "read counters");
    }
    stats[0] = ctx->last_slots;
    stats[1] = c[WP_CNT_LIVE];
    stats[2] = 0;
    for (int k = 1; k < WP_MAX_TIERS; k++) stats[2] += c[2 * k];
    stats[3] = c[WP_CNT_DENSE];
    return WP_OK;
}

wp_status wp_timing_enable(wp_ctx* ctx, int enable) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    collect_timing(ctx);
    for (int k = 0; k < 9; k++) {
        ctx->t_ms[k] = 0.0;
        ctx->t_n[k] = 0;
    }
    ctx->timing = enable != 0;
    return WP_OK;
}

wp_status wp_timing_read(wp_ctx* ctx, int kind, double* total_ms, long long* launches) {
    if (!ctx || kind < 0 || kind > 8) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    collect_timing(ctx);
    if (total_ms) *total_ms = ctx->t_ms[kind];
    if (launches) *launches = ctx->t_n[kind];
    return WP_OK;
}

wp_status wp_engine_replay(wp_ctx* ctx, int reps, double* ms) {
    if (!ctx || reps < 0) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    WP_CUDA(cudaSetDevice(ctx->device), "set device");
    EngineReplay& rp = ctx->replay;
    if (!rp.valid || rp.epoch != g_alloc_epoch) return fail(ctx, WP_ERR_STATE, "no classify batch to replay");
    BatchArgs a = rp.a;
    a.replay_trust = 1;  // the result slots hold results now, not box sizes
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    WP_CUDA(cudaEventCreate(&e0), "event");
    WP_CUDA(cudaEventCreate(&e1), "event");
    WP_CUDA(cudaEventRecord(e0, ctx->stream), "event");
    for (int r = 0; r < reps; r++) {
        // the lists and their counts are as the compaction left them (no
        // pass hands pairs on: each holds only pairs its slab holds); the
        // heads go back to the start
        for (int k = 0; k < rp.nt; k++)
            WP_CUDA(cudaMemsetAsync(rp.cnt + 2 * k + 1, 0, sizeof(int), ctx->stream), "reset head");
        WP_CUDA(cudaMemsetAsync(rp.cnt + WP_CNT_DENSE + 1, 0, sizeof(int), ctx->stream), "reset head");
        for (int k = 0; k < rp.nt; k++) {
            const bool last = k + 1 == rp.nt;
            size_t smem = wp_engine_smem_bytes(rp.half[k], 0, rp.hb, rp.threads[k]);
            WP_CUDA(wp_launch_engine(rp.C, rp.hb, rp.threads[k], smem, ctx->stream, a, rp.list[k], rp.cnt + 2 * k,
                                     rp.cnt + 2 * k + 1, last ? rp.a.ovf : rp.list[k + 1],
                                     last ? rp.cnt + WP_CNT_DENSE : rp.cnt + 2 * (k + 1), rp.half[k], 0, 1, nullptr),
                    "engine pass");
            ctx->launches++;
        }
        if (rp.dense_warps > 0) {
            size_t smem = wp_dense_smem_bytes(rp.T, rp.a.dense_S_cap, rp.C, rp.hb, rp.dense_warps);
            WP_CUDA(wp_launch_dense(rp.hb, rp.dense_warps * 32, smem, ctx->stream, a), "dense launch");
            ctx->launches++;
        }
    }
    WP_CUDA(cudaEventRecord(e1, ctx->stream), "event");
    WP_CUDA(cudaEventSynchronize(e1), "sync");
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    int err = 0;
    WP_CUDA(cudaMemcpy(&err, ctx->d_err.p, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (err) return fail(ctx, WP_ERR_CUDA, "internal: a replayed pass met a pair its slab does not hold");
    return WP_OK;
}

wp_status wp_probe_fp32_peak(wp_ctx* ctx, double* tflops) {
    if (!ctx || !tflops) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int threads = 256, blocks = sms * 8, iters = 4096;
    WP_CUDA(ctx->d_flops.ensure(sizeof(double) * blocks * threads), "alloc probe");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(a, ctx->stream);
        WP_CUDA(wp_launch_fma_probe(blocks, threads, iters, ctx->stream, ctx->d_flops.as<float>()), "probe");
        cudaEventRecord(b, ctx->stream);
        ctx->launches++;
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        double fl = 2.0 * 8.0 * (double)iters * blocks * threads;
        if (rep > 0) best = std::max(best, fl / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *tflops = best;
    return WP_OK;
}

// The device model of a sequencing model for T timesteps (no context state).
wp_status build_dev_model(wp_ctx* ctx, const wp_seq_model* m, int T, DevModel* hp) {
    const int C = m->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS) return fail(ctx, WP_ERR_UNSUPPORTED, "num_channels out of range 1..4");
    if (T < 1 || T > WP_MAX_TIMESTEPS) return fail(ctx, WP_ERR_UNSUPPORTED, "num_timesteps out of range 1..64");
    if (!m->p_bleach || !m->p_dud || !m->bg_sig || !m->mu || !m->sig)
        return fail(ctx, WP_ERR_INVALID, "null per-channel array");
    return wp_fill_dev_model(m, T, hp);
}

wp_status wp_model_upload(wp_ctx* ctx, const wp_seq_model* m, int T) {
    if (!ctx || !m) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    DevModel& h = ctx->hm;
    wp_status st = build_dev_model(ctx, m, T, &h);
    if (st != WP_OK) return st;
    const int C = m->num_channels;
    for (int t = 0; t < T; t++)
        ctx->raw_pdet[t] = m->p_detach + m->p_initial_detach * std::exp(-(double)t * m->p_initial_detach_decay);
    ctx->raw_pf = m->p_edman_failure;
    ctx->raw_pib = m->p_initial_block;
    ctx->raw_pcb = m->p_cyclic_block;
    for (int c = 0; c < C; c++) {
        ctx->raw_pdud[c] = m->p_dud[c];
        ctx->raw_pbleach[c] = m->p_bleach[c];
    }
    WP_CUDA(cudaMemcpyAsync(ctx->d_model.p, &h, sizeof(DevModel), cudaMemcpyHostToDevice, ctx->stream),
            "copy model");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync model");
    ctx->have_model = true;
    ctx->model_version++;
    ctx->plan_C = ctx->plan_T = -1;
    return WP_OK;
}

wp_status wp_peptides_upload(wp_ctx* ctx, const int16_t* dye_seqs, const int32_t* offsets,
                             const int32_t* ids, const int32_t* counts, int P) {
    if (!ctx || P < 0 || (P > 0 && (!offsets || !ids || !counts))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (P > 0 && offsets[0] != 0) return fail(ctx, WP_ERR_INVALID, "offsets[0] must be 0");
    for (int i = 0; i < P; i++)
        if (offsets[i + 1] < offsets[i]) return fail(ctx, WP_ERR_INVALID, "offsets not ascending");
    int n = P > 0 ? offsets[P] : 0;
    if (n > 0 && !dye_seqs) return WP_ERR_INVALID;
    ctx->seqs.assign(dye_seqs, dye_seqs + n);
    ctx->offsets.assign(offsets, offsets + P + 1);
    ctx->ids.assign(ids, ids + P);
    ctx->counts.assign(counts, counts + P);
    ctx->P = P;
    ctx->have_peps = true;
    ctx->pep_version++;
    ctx->plan_C = ctx->plan_T = -1;
    return WP_OK;
}

wp_status wp_hmm_classify(wp_ctx* ctx, const double* rads, int R, double dist_cutoff,
                          const int32_t* cand, const int32_t* cand_off, int32_t* out_id,
                          double* out_score, double* out_total, double* out_log_score) {
    if (!ctx || R < 0 || (R > 0 && (!rads || !out_id || !out_score || !out_total))) return WP_ERR_INVALID;
    if ((cand == nullptr) != (cand_off == nullptr)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    if (ctx->P == 0) return fail(ctx, WP_ERR_INVALID, "no peptides");
    if (cand) {
        if (cand_off[0] != 0) return fail(ctx, WP_ERR_INVALID, "cand_off[0] must be 0");
        for (int r = 0; r < R; r++)
            if (cand_off[r + 1] < cand_off[r]) return fail(ctx, WP_ERR_INVALID, "cand_off not ascending");
    }
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    WP_CUDA(ctx->d_out_id.ensure(sizeof(int32_t) * R), "alloc out");
    WP_CUDA(ctx->d_out_score.ensure(sizeof(double) * R), "alloc out");
    WP_CUDA(ctx->d_out_total.ensure(sizeof(double) * R), "alloc out");
    WP_CUDA(ctx->d_out_log.ensure(sizeof(double) * R), "alloc out");
    st = run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, cand, cand_off, MODE_CLASSIFY, nullptr,
                   ctx->d_out_id.as<int32_t>(), ctx->d_out_score.as<double>(),
                   ctx->d_out_total.as<double>(), ctx->d_out_log.as<double>(), nullptr);
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_id, ctx->d_out_id.p, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    WP_CUDA(cudaMemcpyAsync(out_score, ctx->d_out_score.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    WP_CUDA(cudaMemcpyAsync(out_total, ctx->d_out_total.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    if (out_log_score)
        WP_CUDA(cudaMemcpyAsync(out_log_score, ctx->d_out_log.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    return finish(ctx);
}

wp_status wp_hmm_classify_device(wp_ctx* ctx, const double* d_rads, int R, double dist_cutoff,
                                 int32_t* d_out_id, double* d_out_score, double* d_out_total, int async) {
    if (!ctx || R < 0 || (R > 0 && (!d_rads || !d_out_id || !d_out_score || !d_out_total))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    if (ctx->P == 0) return fail(ctx, WP_ERR_INVALID, "no peptides");
    st = plan_peptides(ctx);
    if (st != WP_OK) return st;
    // CUDA graph of the launch sequence: the second call with the same
    // arguments captures it, later ones replay it (buffers are allocated by
    // the first, uncaptured call).  Not while per-kernel timing is on.
    GraphKey key;
    key.rads = d_rads;
    key.R = R;
    key.cutoff = dist_cutoff;
    key.out[0] = d_out_id;
    key.out[1] = d_out_score;
    key.out[2] = d_out_total;
    key.model_version = ctx->model_version;
    key.pep_version = ctx->pep_version;
    key.alloc_epoch = g_alloc_epoch;
    key.cfg = cfg_for(ctx);
    const bool use_graph = ctx->graphs && !ctx->timing;
    if (use_graph && ctx->gexec && key == ctx->gkey) {
        WP_CUDA(cudaGraphLaunch(ctx->gexec, ctx->stream), "graph launch");
        ctx->launches += ctx->graph_launches;
    } else if (use_graph && key == ctx->gpending) {
        if (ctx->gexec) {
            cudaGraphExecDestroy(ctx->gexec);
            ctx->gexec = nullptr;
        }
        cudaGraph_t g = nullptr;
        WP_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        const long long l0 = ctx->launches;
        st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, nullptr, MODE_CLASSIFY, nullptr, d_out_id,
                       d_out_score, d_out_total, nullptr, nullptr);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
        if (st != WP_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "end capture");
        if (g_alloc_epoch != key.alloc_epoch) {
            // a buffer moved while capturing: run directly this time
            cudaGraphDestroy(g);
            ctx->gpending = GraphKey();
            st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, nullptr, MODE_CLASSIFY, nullptr, d_out_id,
                           d_out_score, d_out_total, nullptr, nullptr);
            if (st != WP_OK) return st;
            return async ? WP_OK : finish(ctx);
        }
        ctx->graph_launches = ctx->launches - l0;
        ce = cudaGraphInstantiate(&ctx->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            ctx->gexec = nullptr;
            return cuda_fail(ctx, ce, "graph instantiate");
        }
        ctx->gkey = key;
        ctx->launches -= ctx->graph_launches;  // counted when they run
        WP_CUDA(cudaGraphLaunch(ctx->gexec, ctx->stream), "graph launch");
        ctx->launches += ctx->graph_launches;
    } else {
        st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, nullptr, MODE_CLASSIFY, nullptr, d_out_id,
                       d_out_score, d_out_total, nullptr, nullptr);
        if (st != WP_OK) return st;
        ctx->gpending = key;
    }
    if (async) return WP_OK;
    return finish(ctx);
}

wp_status wp_ctx_set_graphs(wp_ctx* ctx, int enable) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->graphs = enable != 0;
    return WP_OK;
}

wp_status wp_set_engine_config(wp_ctx* ctx, const int32_t* cfg4) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!cfg4) {
        ctx->force_cfg = false;
        return WP_OK;
    }
    for (int i = 0; i < 4; i += 2)
        if (cfg4[i] < 32 || cfg4[i] > wp_engine_max_threads() || cfg4[i] % 32 || cfg4[i + 1] < 1 || cfg4[i + 1] > 4)
            return fail(ctx, WP_ERR_INVALID, "engine config out of range");
    ctx->forced.t1 = cfg4[0];
    ctx->forced.s1 = cfg4[1];
    ctx->forced.t2 = cfg4[2];
    ctx->forced.s2 = cfg4[3];
    ctx->force_cfg = true;
    return WP_OK;
}

wp_status wp_autotune(wp_ctx* ctx, const double* rads, int R, double dist_cutoff, int32_t* out_cfg4,
                      double* out_best_ms) {
    if (!ctx || R < 1 || !rads) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (ctx->P == 0) return fail(ctx, WP_ERR_INVALID, "no peptides");
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    st = plan_peptides(ctx);
    if (st != WP_OK) return st;
    WP_CUDA(ctx->d_out_id.ensure(sizeof(int) * R), "alloc");
    WP_CUDA(ctx->d_out_score.ensure(sizeof(double) * R), "alloc");
    WP_CUDA(ctx->d_out_total.ensure(sizeof(double) * R), "alloc");
    const bool was_forced = ctx->force_cfg, was_timing = ctx->timing;
    const EngineCfg was = ctx->forced;
    ctx->timing = false;
    EngineCfg best;
    double best_ms = 1e300;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads[2] = {128, 256};
    for (int t1 : threads)
        for (int s1 = 1; s1 <= 4; s1++)
            for (int t2 : threads) {
                EngineCfg c;
                c.t1 = t1;
                c.s1 = s1;
                c.t2 = t2;
                c.s2 = 1;
                const bool hb = ctx->hm.has_block != 0;
                if (slab_half_for(ctx, c.t1, c.s1, hb) < 4 || slab_half_for(ctx, c.t2, c.s2, hb) < 4) continue;
                ctx->forced = c;
                ctx->force_cfg = true;
                double ms_best_c = 1e300;
                bool ok = true;
                for (int rep = 0; rep < 5 && ok; rep++) {  // first run warms up; best of four
                    cudaEventRecord(e0, ctx->stream);
                    if (run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, nullptr, nullptr, MODE_CLASSIFY,
                                  nullptr, ctx->d_out_id.as<int>(), ctx->d_out_score.as<double>(),
                                  ctx->d_out_total.as<double>(), nullptr, nullptr) != WP_OK ||
                        finish(ctx) != WP_OK) {
                        ok = false;
                        break;
                    }
                    cudaEventRecord(e1, ctx->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) ms_best_c = std::min(ms_best_c, (double)ms);
                }
                if (ok && ms_best_c < best_ms) {
                    best_ms = ms_best_c;
                    best = c;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->force_cfg = was_forced;
    ctx->forced = was;
    ctx->timing = was_timing;
    ctx->err.clear();
    if (best_ms >= 1e300) return fail(ctx, WP_ERR_UNSUPPORTED, "no engine configuration ran");
    const long long k = cfg_key(ctx);
    bool found = false;
    for (auto& kv : ctx->tuned)
        if (kv.first == k) {
            kv.second = best;
            found = true;
        }
    if (!found) ctx->tuned.push_back({k, best});
    if (out_cfg4) {
        out_cfg4[0] = best.t1;
        out_cfg4[1] = best.s1;
        out_cfg4[2] = best.t2;
        out_cfg4[3] = best.s2;
    }
    if (out_best_ms) *out_best_ms = best_ms;
    return WP_OK;
}

wp_status wp_hmm_loglik_all(wp_ctx* ctx, const double* rads, int R, double dist_cutoff, double* out_logp) {
    if (!ctx || R < 0 || (R > 0 && (!rads || !out_logp))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (R == 0 || ctx->P == 0) return WP_OK;
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    size_t lbytes = sizeof(double) * (size_t)R * ctx->P;
    WP_CUDA(ctx->d_logp.ensure(lbytes), "alloc logp");
    st = run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, nullptr, nullptr, MODE_LOGP,
                   ctx->d_logp.as<double>(), nullptr, nullptr, nullptr, nullptr, nullptr);
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_logp, ctx->d_logp.p, lbytes, cudaMemcpyDeviceToHost, ctx->stream), "copy logp");
    return finish(ctx);
}

}  // extern "C"

// Error setter for host code in other translation units (wp_fitter.cc).
wp_status wp_internal_fail(wp_ctx* ctx, wp_status code, const char* msg) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    return fail(ctx, code, msg);
}

extern "C" {

wp_status wp_fit_set_kernel(wp_ctx* ctx, int kind) {
    if (!ctx || kind < 0 || kind > 1) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->fit_force_thread = kind == 1;
    return WP_OK;
}

wp_status wp_fit_set_emission(wp_ctx* ctx, int enable) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->fit_emission = enable != 0;
    return WP_OK;
}

wp_status wp_fit_emission_sums(wp_ctx* ctx, wp_emission_sums* out) {
    if (!ctx || !out) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    *out = ctx->fit_emis_last;
    return WP_OK;
}

// Slot layout of wp_fit.cu -> wp_fit_sums.
void fit_sums_from_slots(const double* sums, int T, int C, wp_fit_sums* out) {
    memset(out, 0, sizeof(*out));
    out->p_edman_failure_num = sums[0];
    out->p_edman_failure_den = sums[1];
    out->p_initial_block_num = sums[2];
    out->p_initial_block_den = sums[3];
    out->p_cyclic_block_num = sums[4];
    out->p_cyclic_block_den = sums[5];
    for (int t = 0; t + 1 < T; t++) {
        out->p_detach_x[t] = sums[6 + 2 * t];
        out->p_detach_n[t] = sums[7 + 2 * t];
    }
    for (int c = 0; c < C; c++) {
        const int b = 6 + 2 * (T - 1) + 4 * c;
        out->p_bleach_num[c] = sums[b];
        out->p_bleach_den[c] = sums[b + 1];
        out->p_dud_num[c] = sums[b + 2];
        out->p_dud_den[c] = sums[b + 3];
    }
}

wp_status wp_fit_begin(wp_ctx* ctx, const int16_t* dye_seq, int length, const double* rads, int R) {
    if (!ctx || length < 0 || R < 0 || (length > 0 && !dye_seq) || (R > 0 && !rads)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->have_model) return fail(ctx, WP_ERR_STATE, "model not uploaded");
    const int C = ctx->hm.C, T = ctx->hm.T;
    int cnt[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    for (int k = 0; k < length; k++) {
        if (dye_seq[k] < -1 || dye_seq[k] >= C) return fail(ctx, WP_ERR_INVALID, "dye-seq channel out of range");
        if (dye_seq[k] >= 0) cnt[dye_seq[k]]++;
    }
    ctx->fit_dmax = 0;
    for (int c = 0; c < C; c++) {
        if (cnt[c] > WP_MAX_DYES_PER_CHANNEL) return fail(ctx, WP_ERR_UNSUPPORTED, "more than 15 dyes on a channel");
        ctx->fit_D[c] = cnt[c];
        ctx->fit_dmax = std::max(ctx->fit_dmax, cnt[c]);
    }
    ctx->fit_seq.assign(dye_seq, dye_seq + length);
    ctx->fit_R = R;
    ctx->fit_T = T;
    ctx->fit_C = C;
    const size_t bytes = sizeof(double) * (size_t)R * T * C;
    WP_CUDA(ctx->d_fit_rads.ensure(std::max<size_t>(bytes, 8)), "alloc fit reads");
    if (R > 0) WP_CUDA(cudaMemcpyAsync(ctx->d_fit_rads.p, rads, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy fit reads");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->have_fit = true;
    return WP_OK;
}

wp_status wp_fit_estep(wp_ctx* ctx, wp_fit_sums* out, double* sum_logp, int* num_zero) {
    if (!ctx || !out) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->have_model) return fail(ctx, WP_ERR_STATE, "model not uploaded");
    if (!ctx->have_fit) return fail(ctx, WP_ERR_STATE, "fit not staged (wp_fit_begin)");
    if (ctx->hm.interacting) return fail(ctx, WP_ERR_UNSUPPORTED, "the GPU fit does not support channel interactions");
    const int C = ctx->hm.C, T = ctx->hm.T, R = ctx->fit_R;
    if (C != ctx->fit_C || T != ctx->fit_T)
        return fail(ctx, WP_ERR_STATE, "model channels/timesteps differ from the staged reads");
    const bool hb = ctx->hm.has_block != 0;
    memset(out, 0, sizeof(*out));
    if (sum_logp) *sum_logp = 0.0;
    if (num_zero) *num_zero = 0;
    if (R == 0) return WP_OK;
    // Emission factors of every read, unpruned (run-fit.cc:59), with the
    // HMMFitter's max_num_dyes (fitters/hmm-fitter.cc:30-52).
    const int W = ctx->fit_dmax + 1;
    const int entries = T * C * W;
    WP_CUDA(ctx->d_fit_lo.ensure((size_t)R * T * C), "alloc");
    WP_CUDA(ctx->d_fit_hi.ensure((size_t)R * T * C), "alloc");
    WP_CUDA(ctx->d_fit_tab.ensure(sizeof(EmitEntry) * (size_t)R * entries), "alloc fit table");
    {
        long n = (long)R * T;
        TimedLaunch tl(ctx, 1);
        wp_prep_reads_kernel<<<(int)((n + 127) / 128), 128, 0, ctx->stream>>>(
                ctx->d_model.as<DevModel>(), ctx->d_fit_rads.as<double>(), R, (unsigned)ctx->fit_dmax, DBL_MAX,
                ctx->d_fit_lo.as<uint8_t>(), ctx->d_fit_hi.as<uint8_t>(), ctx->d_fit_tab.as<EmitEntry>(), entries);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "fit prep launch");
    }
    int S = 1;
    for (int c = 0; c < C; c++) S *= ctx->fit_D[c] + 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const bool emis = ctx->fit_emission;
    const int nslots = wp_fit_nslots(T, C, emis);
    // CTA-per-read kernel when a read's vectors fit shared memory, else the
    // thread-per-read kernel over a global slab.
    const size_t cta_smem = wp_fit_cta_smem_bytes(T, C, S, hb, emis);
    // (the kernel also holds the binomial tables in static shared memory)
    const int cta_per_sm = (long)cta_smem + (long)sizeof(SmemModel) <= (long)ctx->smem_optin
                                   ? wp_fit_cta_ctas_per_sm(hb, cta_smem)
                                   : 0;
    const bool use_cta = cta_per_sm > 0 && !ctx->fit_force_thread;
    const int threads = 128;
    int grid = 0;
    long nth = 0, per = 0, ck_stride = 0;
    if (use_cta) {
        grid = (int)std::min<long>((long)R, (long)sms * cta_per_sm);
        nth = grid;
        ck_stride = wp_fit_cta_ckpt_floats(T, S, hb);
        WP_CUDA(ctx->d_fit_scratch.ensure(sizeof(float) * (size_t)grid * ck_stride), "alloc fit checkpoints");
    } else {
        long want = std::min<long>((long)R, (long)sms * 4 * threads);
        per = wp_fit_floats_per_thread(T, C, S, hb);
        // keep the scratch under 16 GiB
        while (want > threads && (double)want * per * 4.0 > 16.0 * (1u << 30)) want /= 2;
        grid = (int)((want + threads - 1) / threads);
        nth = (long)grid * threads;
        WP_CUDA(ctx->d_fit_scratch.ensure(sizeof(float) * (size_t)nth * per), "alloc fit scratch");
    }
    WP_CUDA(ctx->d_fit_sums.ensure(sizeof(double) * (size_t)nth * nslots), "alloc fit sums");
    WP_CUDA(ctx->d_fit_out.ensure(sizeof(double) * nslots), "alloc fit sums");
    WP_CUDA(ctx->d_fit_logp.ensure(sizeof(double) * R), "alloc fit logp");
    FitArgs fa;
    memset(&fa, 0, sizeof(fa));
    fa.model = ctx->d_model.as<DevModel>();
    fa.rads = ctx->d_fit_rads.as<double>();
    fa.R = R;
    for (int c = 0; c < C; c++) fa.D[c] = ctx->fit_D[c];
    {
        int rem[WP_MAX_CHANNELS];
        for (int c = 0; c < WP_MAX_CHANNELS; c++) rem[c] = ctx->fit_D[c];
        const int len = (int)ctx->fit_seq.size();
        for (int e = 0; e < WP_MAX_TIMESTEPS; e++) {
            int d = e < len ? ctx->fit_seq[e] : -1;
            fa.dye[e] = (int8_t)d;
            fa.tot[e] = (uint8_t)(d >= 0 ? rem[d] : 0);  // DyeTrack(e, d)
            if (d >= 0) rem[d]--;
        }
    }
    fa.tab = ctx->d_fit_tab.as<EmitEntry>();
    fa.W = W;
    fa.scratch = ctx->d_fit_scratch.as<float>();
    fa.vec_floats = per;
    fa.sums = ctx->d_fit_sums.as<double>();
    fa.logp = ctx->d_fit_logp.as<double>();
    fa.nslots = nslots;
    fa.emission = emis ? 1 : 0;
    {
        TimedLaunch tl(ctx, 0);
        if (use_cta)
            WP_CUDA(wp_launch_fit_cta(hb, grid, cta_smem, ctx->stream, fa, ctx->d_fit_scratch.as<float>(), ck_stride),
                    "fit E-step launch");
        else
            WP_CUDA(wp_launch_fit_estep(hb, grid, threads, ctx->stream, fa), "fit E-step launch");
        ctx->launches++;
    }
    wp_fit_reduce_kernel<<<(nslots + 63) / 64, 64, 0, ctx->stream>>>(fa.sums, nth, nslots, ctx->d_fit_out.as<double>());
    ctx->launches++;
    WP_CUDA(cudaGetLastError(), "fit reduce launch");
    std::vector<double> sums(nslots), lp(R);
    WP_CUDA(cudaMemcpyAsync(sums.data(), ctx->d_fit_out.p, sizeof(double) * nslots, cudaMemcpyDeviceToHost, ctx->stream), "copy sums");
    WP_CUDA(cudaMemcpyAsync(lp.data(), ctx->d_fit_logp.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy logp");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    fit_sums_from_slots(sums.data(), T, C, out);
    memset(&ctx->fit_emis_last, 0, sizeof(ctx->fit_emis_last));
    if (emis) {
        // slots after the rates: [kind][c][n], kind w / x / xx (wp_fit.cu)
        const int base = 6 + 2 * (T - 1) + 4 * C, N = WP_MAX_DYES_PER_CHANNEL + 1;
        for (int c = 0; c < C; c++)
            for (int n = 0; n < N; n++) {
                ctx->fit_emis_last.w[c][n] = sums[base + (0 * C + c) * N + n];
                ctx->fit_emis_last.x[c][n] = sums[base + (1 * C + c) * N + n];
                ctx->fit_emis_last.xx[c][n] = sums[base + (2 * C + c) * N + n];
            }
    }
    double sl = 0.0;
    int nz = 0;
    for (int r = 0; r < R; r++) {
        if (std::isfinite(lp[r])) sl += lp[r];
        else nz++;
    }
    if (sum_logp) *sum_logp = sl;
    if (num_zero) *num_zero = nz;
    return WP_OK;
}

wp_status wp_fit_estep_batch(wp_ctx* ctx, const wp_seq_model* models, int B, const int32_t* read_idx, int Rb,
                             wp_fit_sums* out, double* sum_logp, int* num_zero) {
    if (!ctx || !models || B < 1 || Rb < 0 || !out || (Rb > 0 && !read_idx)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->have_fit) return fail(ctx, WP_ERR_STATE, "fit not staged (wp_fit_begin)");
    const int C = ctx->fit_C, T = ctx->fit_T, R = ctx->fit_R;
    if (ctx->fit_emission) return fail(ctx, WP_ERR_UNSUPPORTED, "batched E-steps keep the emission parameters fixed");
    // the instances' models: same shape and emission parameters as the staged
    // fit (they share the reads' emission factors), no interactions
    std::vector<DevModel> hm(B);
    for (int b = 0; b < B; b++) {
        if (models[b].num_channels != C) return fail(ctx, WP_ERR_INVALID, "model channels differ from the staged reads");
        wp_status st = build_dev_model(ctx, &models[b], T, &hm[b]);
        if (st != WP_OK) return st;
        if (hm[b].interacting) return fail(ctx, WP_ERR_UNSUPPORTED, "the GPU fit does not support channel interactions");
        for (int c = 0; c < C; c++)
            if (hm[b].mu[c] != hm[0].mu[c] || hm[b].sig[c] != hm[0].sig[c] || hm[b].bg_sig[c] != hm[0].bg_sig[c])
                return fail(ctx, WP_ERR_INVALID, "batched instances need the same emission parameters");
        if (hm[b].has_block != hm[0].has_block)
            return fail(ctx, WP_ERR_UNSUPPORTED, "batched instances must all block or all not block");
    }
    for (long i = 0; i < (long)B * Rb; i++)
        if (read_idx[i] < 0 || read_idx[i] >= R) return fail(ctx, WP_ERR_INVALID, "read index out of range");
    for (int b = 0; b < B; b++) {
        memset(&out[b], 0, sizeof(out[b]));
        if (sum_logp) sum_logp[b] = 0.0;
        if (num_zero) num_zero[b] = 0;
    }
    if (Rb == 0 || R == 0) return WP_OK;
    const bool hb = hm[0].has_block != 0;
    // emission factors of the staged reads, from the shared emission model
    ctx->hm = hm[0];
    WP_CUDA(cudaMemcpyAsync(ctx->d_model.p, &hm[0], sizeof(DevModel), cudaMemcpyHostToDevice, ctx->stream), "copy model");
    ctx->model_version++;
    const int W = ctx->fit_dmax + 1;
    const int entries = T * C * W;
    WP_CUDA(ctx->d_fit_lo.ensure((size_t)R * T * C), "alloc");
    WP_CUDA(ctx->d_fit_hi.ensure((size_t)R * T * C), "alloc");
    WP_CUDA(ctx->d_fit_tab.ensure(sizeof(EmitEntry) * (size_t)R * entries), "alloc fit table");
    {
        long n = (long)R * T;
        TimedLaunch tl(ctx, 1);
        wp_prep_reads_kernel<<<(int)((n + 127) / 128), 128, 0, ctx->stream>>>(
                ctx->d_model.as<DevModel>(), ctx->d_fit_rads.as<double>(), R, (unsigned)ctx->fit_dmax, DBL_MAX,
                ctx->d_fit_lo.as<uint8_t>(), ctx->d_fit_hi.as<uint8_t>(), ctx->d_fit_tab.as<EmitEntry>(), entries);
        ctx->launches++;
        WP_CUDA(cudaGetLastError(), "fit prep launch");
    }
    int S = 1;
    for (int c = 0; c < C; c++) S *= ctx->fit_D[c] + 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int nslots = wp_fit_nslots(T, C, false);
    const size_t cta_smem = wp_fit_cta_smem_bytes(T, C, S, hb, false);
    const int cta_per_sm = (long)cta_smem + (long)sizeof(SmemModel) <= (long)ctx->smem_optin
                                   ? wp_fit_cta_ctas_per_sm(hb, cta_smem)
                                   : 0;
    if (cta_per_sm <= 0) return fail(ctx, WP_ERR_UNSUPPORTED, "batched E-steps need the CTA-per-read kernel");
    // CTAs per instance: the device's resident CTAs shared out (rounded down,
    // so that all CTAs are resident in one wave), at most one per read
    const int G = (int)std::max<long>(1, std::min<long>((long)Rb, ((long)sms * cta_per_sm) / B));
    const long grid = (long)G * B;
    if (grid > INT32_MAX) return fail(ctx, WP_ERR_UNSUPPORTED, "too many batched instances");
    const long ck_stride = wp_fit_cta_ckpt_floats(T, S, hb);
    WP_CUDA(ctx->d_fit_scratch.ensure(sizeof(float) * (size_t)grid * ck_stride), "alloc fit checkpoints");
    WP_CUDA(ctx->d_fit_sums.ensure(sizeof(double) * (size_t)grid * nslots), "alloc fit sums");
    WP_CUDA(ctx->d_fit_logp.ensure(sizeof(double) * (size_t)B * Rb), "alloc fit logp");
    WP_CUDA(ctx->d_boot_models.ensure(sizeof(DevModel) * B), "alloc models");
    WP_CUDA(ctx->d_boot_idx.ensure(sizeof(int) * (size_t)B * Rb), "alloc read lists");
    WP_CUDA(cudaMemcpyAsync(ctx->d_boot_models.p, hm.data(), sizeof(DevModel) * B, cudaMemcpyHostToDevice,
                            ctx->stream), "copy models");
    WP_CUDA(cudaMemcpyAsync(ctx->d_boot_idx.p, read_idx, sizeof(int) * (size_t)B * Rb, cudaMemcpyHostToDevice,
                            ctx->stream), "copy read lists");
    FitArgs fa;
    memset(&fa, 0, sizeof(fa));
    fa.model = ctx->d_boot_models.as<DevModel>();
    fa.rads = ctx->d_fit_rads.as<double>();
    fa.R = Rb;
    for (int c = 0; c < C; c++) fa.D[c] = ctx->fit_D[c];
    {
        int rem[WP_MAX_CHANNELS];
        for (int c = 0; c < WP_MAX_CHANNELS; c++) rem[c] = ctx->fit_D[c];
        const int len = (int)ctx->fit_seq.size();
        for (int e = 0; e < WP_MAX_TIMESTEPS; e++) {
            int d = e < len ? ctx->fit_seq[e] : -1;
            fa.dye[e] = (int8_t)d;
            fa.tot[e] = (uint8_t)(d >= 0 ? rem[d] : 0);  // DyeTrack(e, d)
            if (d >= 0) rem[d]--;
        }
    }
    fa.tab = ctx->d_fit_tab.as<EmitEntry>();
    fa.W = W;
    fa.scratch = ctx->d_fit_scratch.as<float>();
    fa.sums = ctx->d_fit_sums.as<double>();
    fa.logp = ctx->d_fit_logp.as<double>();
    fa.nslots = nslots;
    fa.emission = 0;
    fa.inst_ctas = G;
    fa.read_idx = ctx->d_boot_idx.as<int>();
    {
        TimedLaunch tl(ctx, 0);
        WP_CUDA(wp_launch_fit_cta(hb, (int)grid, cta_smem, ctx->stream, fa, ctx->d_fit_scratch.as<float>(), ck_stride),
                "fit E-step launch");
        ctx->launches++;
    }
    // per-CTA sums [nslots][grid]; each instance's CTAs summed in CTA order
    std::vector<double> part((size_t)nslots * grid), lp((size_t)B * Rb);
    WP_CUDA(cudaMemcpyAsync(part.data(), ctx->d_fit_sums.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                            ctx->stream), "copy sums");
    WP_CUDA(cudaMemcpyAsync(lp.data(), ctx->d_fit_logp.p, sizeof(double) * lp.size(), cudaMemcpyDeviceToHost,
                            ctx->stream), "copy logp");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    std::vector<double> sums(nslots);
    for (int b = 0; b < B; b++) {
        for (int k = 0; k < nslots; k++) {
            double acc = 0.0;
            for (int g = 0; g < G; g++) acc += part[(size_t)k * grid + (size_t)b * G + g];
            sums[k] = acc;
        }
        fit_sums_from_slots(sums.data(), T, C, &out[b]);
        double sl = 0.0;
        int nz = 0;
        for (int r = 0; r < Rb; r++) {
            const double v = lp[(size_t)b * Rb + r];
            if (std::isfinite(v)) sl += v;
            else nz++;
        }
        if (sum_logp) sum_logp[b] = sl;
        if (num_zero) num_zero[b] = nz;
    }
    return WP_OK;
}

// Validates and installs a dye-track set as the kNN training set (caller
// holds the context lock).
wp_status nn_install(wp_ctx* ctx, const int16_t* counts, int N, int T, int C, const int32_t* src_off,
                     const int32_t* src_id, const int32_t* src_count, const int32_t* src_hits) {
    if (C < 1 || C > WP_MAX_CHANNELS || T < 1 || T > WP_MAX_TIMESTEPS)
        return fail(ctx, WP_ERR_UNSUPPORTED, "dye-track shape out of range");
    if (nn_padded_dim(T * C) < 0) return fail(ctx, WP_ERR_UNSUPPORTED, "kNN needs timesteps x channels <= 64");
    const int S = N > 0 ? src_off[N] : 0;
    if (N > 0 && src_off[0] != 0) return fail(ctx, WP_ERR_INVALID, "src_off[0] must be 0");
    if (S > 0 && (!src_id || !src_count || !src_hits)) return WP_ERR_INVALID;
    std::vector<int> ehits(std::max(N, 1), 0);
    for (int e = 0; e < N; e++) {
        if (src_off[e + 1] < src_off[e]) return fail(ctx, WP_ERR_INVALID, "src_off not ascending");
        long long hsum = 0;
        for (int s2 = src_off[e]; s2 < src_off[e + 1]; s2++) {
            if (src_hits[s2] < 0 || src_count[s2] < 0) return fail(ctx, WP_ERR_INVALID, "negative hits or count");
            hsum += src_hits[s2];
        }
        if (hsum < 1 || hsum > INT32_MAX) return fail(ctx, WP_ERR_INVALID, "every dye-track needs 1..2^31-1 hits");
        ehits[e] = (int)hsum;
    }
    ctx->nn_hits_total = 0;
    for (int e = 0; e < N; e++) ctx->nn_hits_total += ehits[e];
    ctx->nn_counts.assign(counts, counts + (size_t)N * T * C);
    ctx->nn_src_off.assign(src_off, src_off + (N > 0 ? N + 1 : 0));
    ctx->nn_src_id.assign(src_id, src_id + S);
    ctx->nn_src_count.assign(src_count, src_count + S);
    ctx->nn_src_hits.assign(src_hits, src_hits + S);
    ctx->nn_uniq = ctx->nn_src_id;
    std::sort(ctx->nn_uniq.begin(), ctx->nn_uniq.end());
    ctx->nn_uniq.erase(std::unique(ctx->nn_uniq.begin(), ctx->nn_uniq.end()), ctx->nn_uniq.end());
    ctx->nn_N = N;
    ctx->nn_T = T;
    ctx->nn_C = C;
    ctx->nn_U = (int)ctx->nn_uniq.size();
    WP_CUDA(ctx->d_nn_dense_id.ensure(sizeof(int) * std::max(ctx->nn_U, 1)), "alloc");
    if (ctx->nn_U > 0)
        WP_CUDA(cudaMemcpyAsync(ctx->d_nn_dense_id.p, ctx->nn_uniq.data(), sizeof(int) * ctx->nn_U, cudaMemcpyHostToDevice, ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->have_tracks = true;
    ctx->nn_coords_version = -1;
    ctx->nn_tree_k = -1;
    ctx->nn_pep_version = -1;
    return WP_OK;
}

wp_status wp_nn_set_selection(wp_ctx* ctx, int selection) {
    if (!ctx || (selection != WP_NN_KDTREE && selection != WP_NN_PREFIX)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->nn_selection = selection;
    return WP_OK;
}

wp_status wp_nn_kd_tree_order(const double* coords, int N, int D, int k, int32_t* perm, int* out_num_nodes) {
    if (N < 0 || D < 1 || D > 64 || (N > 0 && (!coords || !perm))) return WP_ERR_INVALID;
    std::vector<int> p;
    std::vector<KDNode> nodes;
    int depth = 0;
    if (wp_kdtree_build(coords, N, D, k, &p, &nodes, &depth) != 0) return WP_ERR_UNSUPPORTED;
    for (int i = 0; i < N; i++) perm[i] = p[i];
    if (out_num_nodes) *out_num_nodes = (int)nodes.size();
    return WP_OK;
}

wp_status wp_nn_tracks_upload(wp_ctx* ctx, const int16_t* counts, int N, int T, int C, const int32_t* src_off,
                              const int32_t* src_id, const int32_t* src_count, const int32_t* src_hits) {
    if (!ctx || N < 0 || (N > 0 && (!counts || !src_off))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return nn_install(ctx, counts, N, T, C, src_off, src_id, src_count, src_hits);
}

// ---- dye-track generation and dedup ---------------------------------------

namespace {

int field_bits(int most) {
    int b = 1;
    while ((1 << b) <= most) b++;
    return b;
}

// Runs the dedup of n instances already on the device (d_dd_in as int16, or
// in_u8 with per-instance peptide indices) and keeps the result.
wp_status dedup_run(wp_ctx* ctx, int n, int T, int C, int bits, const uint8_t* in_u8, const int* pep,
                    bool drop_zero, long long id_min, long long id_max) {
    const int TC = T * C, k = 64 / bits, W = (TC + k - 1) / k;
    // fold the id offset into the last word when it fits below the fields
    const int last_bits = bits * (TC - (W - 1) * k);
    int id_bits = 0;
    while (id_bits < 33 && ((id_max - id_min) >> id_bits) != 0) id_bits++;
    const bool fold = last_bits + id_bits <= 64;
    const size_t nn = (size_t)std::max(n, 1);
    WP_CUDA(ctx->d_dd_words.ensure(sizeof(uint64_t) * W * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_k0.ensure(sizeof(uint64_t) * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_k1.ensure(sizeof(uint64_t) * nn), "alloc dedup");
    for (DevBuf* b : {&ctx->d_dd_p0, &ctx->d_dd_p1, &ctx->d_dd_id, &ctx->d_dd_cnt, &ctx->d_dd_ft, &ctx->d_dd_fs,
                      &ctx->d_dd_st, &ctx->d_dd_ss, &ctx->d_dd_start, &ctx->d_dd_sid, &ctx->d_dd_scnt,
                      &ctx->d_dd_hits})
        WP_CUDA(b->ensure(sizeof(int) * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_off.ensure(sizeof(int) * (nn + 1)), "alloc dedup");
    WP_CUDA(ctx->d_dd_counts.ensure(sizeof(int16_t) * TC * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_sizes.ensure(sizeof(int) * 2), "alloc dedup");
    const size_t tb = wp_dedup_temp_bytes(n);
    WP_CUDA(ctx->d_dd_temp.ensure(tb), "alloc dedup");
    ctx->dd_valid = false;
    int sizes[2] = {0, 0};
    if (n > 0) {
        DedupArgs a;
        memset(&a, 0, sizeof(a));
        a.n = n;
        a.TC = TC;
        a.bits = bits;
        a.W = W;
        a.drop_zero = drop_zero ? 1 : 0;
        a.fold_id = fold ? 1 : 0;
        a.id_shift = 64 - last_bits - id_bits;
        a.id_min = id_min;
        a.last_mask = ~0ull << (64 - last_bits);
        a.in_u8 = in_u8;
        a.in_i16 = in_u8 ? nullptr : ctx->d_dd_in.as<int16_t>();
        a.pep = pep;
        a.pep_ids = ctx->d_sim_ids.as<int>();
        a.pep_cnts = ctx->d_sim_cnts.as<int>();
        a.inst_id = ctx->d_dd_id.as<int>();
        a.inst_cnt = ctx->d_dd_cnt.as<int>();
        a.words = ctx->d_dd_words.as<uint64_t>();
        a.keys0 = ctx->d_dd_k0.as<uint64_t>();
        a.keys1 = ctx->d_dd_k1.as<uint64_t>();
        a.perm0 = ctx->d_dd_p0.as<int>();
        a.perm1 = ctx->d_dd_p1.as<int>();
        a.flag_t = ctx->d_dd_ft.as<int>();
        a.flag_s = ctx->d_dd_fs.as<int>();
        a.scan_t = ctx->d_dd_st.as<int>();
        a.scan_s = ctx->d_dd_ss.as<int>();
        a.start = ctx->d_dd_start.as<int>();
        a.temp = ctx->d_dd_temp.p;
        a.temp_bytes = tb;
        a.out_counts = ctx->d_dd_counts.as<int16_t>();
        a.out_src_off = ctx->d_dd_off.as<int>();
        a.out_src_id = ctx->d_dd_sid.as<int>();
        a.out_src_count = ctx->d_dd_scnt.as<int>();
        a.out_src_hits = ctx->d_dd_hits.as<int>();
        a.out_sizes = ctx->d_dd_sizes.as<int>();
        int nl = 0;
        {
            TimedLaunch tl(ctx, 7);
            WP_CUDA(wp_launch_dedup(a, ctx->stream, &nl), "dedup launch");
        }
        ctx->launches += nl;
        WP_CUDA(cudaMemcpyAsync(sizes, a.out_sizes, sizeof(sizes), cudaMemcpyDeviceToHost, ctx->stream), "copy");
    } else {
        WP_CUDA(cudaMemsetAsync(ctx->d_dd_off.p, 0, sizeof(int), ctx->stream), "clear");
    }
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync dedup");
    ctx->dd_U = sizes[0];
    ctx->dd_S = sizes[1];
    ctx->dd_T = T;
    ctx->dd_C = C;
    ctx->dd_valid = true;
    return WP_OK;
}

}  // namespace

wp_status wp_dedup_dye_tracks(wp_ctx* ctx, const int16_t* counts, const int32_t* ids, const int32_t* src_counts,
                              int N, int T, int C, int* out_num_tracks, int* out_num_sources) {
    if (!ctx || N < 0 || (N > 0 && (!counts || !ids || !src_counts))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (C < 1 || C > WP_MAX_CHANNELS || T < 1 || T > WP_MAX_TIMESTEPS)
        return fail(ctx, WP_ERR_UNSUPPORTED, "dye-track shape out of range");
    const size_t total = (size_t)N * T * C;
    const size_t nn = (size_t)std::max(N, 1);
    WP_CUDA(ctx->d_dd_in.ensure(sizeof(int16_t) * std::max<size_t>(total, 1)), "alloc dedup");
    WP_CUDA(ctx->d_dd_id.ensure(sizeof(int) * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_cnt.ensure(sizeof(int) * nn), "alloc dedup");
    WP_CUDA(ctx->d_dd_sizes.ensure(sizeof(int) * 2), "alloc dedup");
    int bits = 1;
    if (N > 0) {
        WP_CUDA(cudaMemcpyAsync(ctx->d_dd_in.p, counts, sizeof(int16_t) * total, cudaMemcpyHostToDevice, ctx->stream),
                "copy");
        WP_CUDA(cudaMemcpyAsync(ctx->d_dd_id.p, ids, sizeof(int) * N, cudaMemcpyHostToDevice, ctx->stream), "copy");
        WP_CUDA(cudaMemcpyAsync(ctx->d_dd_cnt.p, src_counts, sizeof(int) * N, cudaMemcpyHostToDevice, ctx->stream),
                "copy");
        WP_CUDA(wp_launch_dedup_range(ctx->d_dd_in.as<int16_t>(), total, ctx->d_dd_sizes.as<int>(), ctx->stream),
                "dedup range");
        ctx->launches++;
        int mm[2];
        WP_CUDA(cudaMemcpyAsync(mm, ctx->d_dd_sizes.p, sizeof(mm), cudaMemcpyDeviceToHost, ctx->stream), "copy");
        WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        if (mm[0] < 0) return fail(ctx, WP_ERR_INVALID, "negative dye count");
        bits = field_bits(mm[1]);
    }
    long long id_min = 0, id_max = 0;
    if (N > 0) {
        auto mm = std::minmax_element(ids, ids + N);
        id_min = *mm.first;
        id_max = *mm.second;
    }
    wp_status st = dedup_run(ctx, N, T, C, bits, nullptr, nullptr, false, id_min, id_max);
    if (st != WP_OK) return st;
    if (out_num_tracks) *out_num_tracks = ctx->dd_U;
    if (out_num_sources) *out_num_sources = ctx->dd_S;
    return WP_OK;
}

wp_status wp_simulate_dye_tracks(wp_ctx* ctx, int per_peptide, unsigned long long seed, int* out_num_tracks,
                                 int* out_num_sources, uint8_t* out_instance_tracks, int32_t* out_instance_pep) {
    if (!ctx || per_peptide < 0) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    long long copies = 0;
    for (int i = 0; i < ctx->P; i++) {
        if (ctx->counts[i] < 0) return fail(ctx, WP_ERR_INVALID, "negative peptide count");
        copies += ctx->counts[i];
    }
    const long long n64 = copies * per_peptide;
    if (n64 > INT32_MAX) return fail(ctx, WP_ERR_UNSUPPORTED, "more than 2^31-1 dye-tracks to generate");
    const int n = (int)n64;
    const int T = ctx->hm.T, C = ctx->hm.C, TC = T * C;
    if (n > 0) {
        WP_CUDA(ctx->d_sim_pep.ensure(sizeof(int) * n), "alloc");
        WP_CUDA(ctx->d_sim_tracks.ensure((size_t)n * TC), "alloc");
        st = sim_device(ctx, n, seed, nullptr, nullptr, ctx->d_sim_pep.as<int>(), ctx->d_sim_tracks.as<uint8_t>(),
                        per_peptide);
        if (st != WP_OK) return st;
        if (ctx->sim_max_dyes > 255) return fail(ctx, WP_ERR_UNSUPPORTED, "more than 255 dyes of one channel");
    }
    long long id_min = 0, id_max = 0;
    if (ctx->P > 0) {
        auto mm = std::minmax_element(ctx->ids.begin(), ctx->ids.end());
        id_min = *mm.first;
        id_max = *mm.second;
    }
    st = dedup_run(ctx, n, T, C, field_bits(ctx->sim_max_dyes), ctx->d_sim_tracks.as<uint8_t>(),
                   ctx->d_sim_pep.as<int>(), true, id_min, id_max);
    if (st != WP_OK) return st;
    if (n > 0 && out_instance_tracks)
        WP_CUDA(cudaMemcpyAsync(out_instance_tracks, ctx->d_sim_tracks.p, (size_t)n * TC, cudaMemcpyDeviceToHost,
                                ctx->stream), "copy");
    if (n > 0 && out_instance_pep)
        WP_CUDA(cudaMemcpyAsync(out_instance_pep, ctx->d_sim_pep.p, sizeof(int) * n, cudaMemcpyDeviceToHost,
                                ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    if (out_num_tracks) *out_num_tracks = ctx->dd_U;
    if (out_num_sources) *out_num_sources = ctx->dd_S;
    return WP_OK;
}

wp_status wp_dye_tracks_download(wp_ctx* ctx, int16_t* counts, int32_t* src_off, int32_t* src_id,
                                 int32_t* src_count, int32_t* src_hits) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->dd_valid) return fail(ctx, WP_ERR_INVALID, "no dye-track set to download");
    const int U = ctx->dd_U, S = ctx->dd_S;
    if (!src_off || (U > 0 && !counts) || (S > 0 && (!src_id || !src_count || !src_hits))) return WP_ERR_INVALID;
    const size_t TC = (size_t)ctx->dd_T * ctx->dd_C;
    if (U > 0)
        WP_CUDA(cudaMemcpyAsync(counts, ctx->d_dd_counts.p, sizeof(int16_t) * TC * U, cudaMemcpyDeviceToHost,
                                ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(src_off, ctx->d_dd_off.p, sizeof(int) * (U + 1), cudaMemcpyDeviceToHost, ctx->stream),
            "copy");
    if (S > 0) {
        WP_CUDA(cudaMemcpyAsync(src_id, ctx->d_dd_sid.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        WP_CUDA(cudaMemcpyAsync(src_count, ctx->d_dd_scnt.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream),
                "copy");
        WP_CUDA(cudaMemcpyAsync(src_hits, ctx->d_dd_hits.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream),
                "copy");
    }
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return WP_OK;
}

wp_status wp_dye_tracks_to_nn(wp_ctx* ctx) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->dd_valid) return fail(ctx, WP_ERR_INVALID, "no dye-track set to install");
    const int U = ctx->dd_U, S = ctx->dd_S;
    const size_t TC = (size_t)ctx->dd_T * ctx->dd_C;
    std::vector<int16_t> counts(std::max<size_t>(TC * U, 1));
    std::vector<int32_t> off(U + 1), id(std::max(S, 1)), cnt(std::max(S, 1)), hits(std::max(S, 1));
    if (U > 0)
        WP_CUDA(cudaMemcpyAsync(counts.data(), ctx->d_dd_counts.p, sizeof(int16_t) * TC * U, cudaMemcpyDeviceToHost,
                                ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(off.data(), ctx->d_dd_off.p, sizeof(int) * (U + 1), cudaMemcpyDeviceToHost, ctx->stream),
            "copy");
    if (S > 0) {
        WP_CUDA(cudaMemcpyAsync(id.data(), ctx->d_dd_sid.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream),
                "copy");
        WP_CUDA(cudaMemcpyAsync(cnt.data(), ctx->d_dd_scnt.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream),
                "copy");
        WP_CUDA(cudaMemcpyAsync(hits.data(), ctx->d_dd_hits.p, sizeof(int) * S, cudaMemcpyDeviceToHost, ctx->stream),
                "copy");
    }
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return nn_install(ctx, counts.data(), U, ctx->dd_T, ctx->dd_C, off.data(), id.data(), cnt.data(), hits.data());
}

wp_status wp_nn_classify(wp_ctx* ctx, const double* rads, int R, int k, double sig, int h, int32_t* out_ncand,
                         int32_t* out_cand_id, double* out_cand_score, double* out_total) {
    if (!ctx || R < 0 || (R > 0 && (!rads || !out_ncand || !out_cand_id || !out_cand_score || !out_total)))
        return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = nn_check(ctx, k, sig, h);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    st = nn_run(ctx, ctx->d_rads.as<double>(), R, k, sig, h, false);
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_ncand, ctx->d_nn_ncand.p, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_total, ctx->d_nn_total.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_cand_id, ctx->d_nn_cand_id.p, sizeof(int) * (size_t)R * h, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_cand_score, ctx->d_nn_cand_score.p, sizeof(double) * (size_t)R * h, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return WP_OK;
}

wp_status wp_hybrid_classify(wp_ctx* ctx, const double* rads, int R, int k, double sig, int h, double dist_cutoff,
                             int32_t* out_id, double* out_score, double* out_total) {
    if (!ctx || R < 0 || (R > 0 && (!rads || !out_id || !out_score || !out_total))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = hybrid_check(ctx, k, sig, h);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    WP_CUDA(ctx->d_out_id.ensure(sizeof(int) * R), "alloc outputs");
    WP_CUDA(ctx->d_out_score.ensure(sizeof(double) * R), "alloc outputs");
    WP_CUDA(ctx->d_out_total.ensure(sizeof(double) * R), "alloc outputs");
    st = hybrid_run(ctx, ctx->d_rads.as<double>(), R, k, sig, h, dist_cutoff, ctx->d_out_id.as<int>(),
                    ctx->d_out_score.as<double>(), ctx->d_out_total.as<double>());
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_id, ctx->d_out_id.p, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_score, ctx->d_out_score.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_total, ctx->d_out_total.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    return finish(ctx);
}

wp_status wp_hybrid_classify_device(wp_ctx* ctx, const double* d_rads, int R, int k, double sig, int h,
                                    double dist_cutoff, int32_t* d_out_id, double* d_out_score,
                                    double* d_out_total) {
    if (!ctx || R < 0 || (R > 0 && (!d_rads || !d_out_id || !d_out_score || !d_out_total))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = hybrid_check(ctx, k, sig, h);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    st = hybrid_run(ctx, d_rads, R, k, sig, h, dist_cutoff, d_out_id, d_out_score, d_out_total);
    if (st != WP_OK) return st;
    return finish(ctx);
}

wp_status wp_simulate_reads(wp_ctx* ctx, int R, unsigned long long seed, double* out_rads, int32_t* out_pep,
                            uint8_t* out_tracks) {
    if (!ctx || R < 0 || (R > 0 && (!out_rads || !out_pep))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (ctx->P == 0) return fail(ctx, WP_ERR_INVALID, "no peptides to simulate");
    if (R == 0) return WP_OK;
    const size_t TC = (size_t)ctx->hm.T * ctx->hm.C;
    WP_CUDA(ctx->d_sim_rads.ensure(sizeof(double) * R * TC), "alloc");
    WP_CUDA(ctx->d_sim_pep.ensure(sizeof(int) * R), "alloc");
    if (out_tracks) WP_CUDA(ctx->d_sim_tracks.ensure(R * TC), "alloc");
    st = sim_device(ctx, R, seed, nullptr, ctx->d_sim_rads.as<double>(), ctx->d_sim_pep.as<int>(),
                    out_tracks ? ctx->d_sim_tracks.as<uint8_t>() : nullptr);
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_rads, ctx->d_sim_rads.p, sizeof(double) * R * TC, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaMemcpyAsync(out_pep, ctx->d_sim_pep.p, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (out_tracks)
        WP_CUDA(cudaMemcpyAsync(out_tracks, ctx->d_sim_tracks.p, R * TC, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return WP_OK;
}

wp_status wp_dev_gemm_bf16(const void* A, int lda, const void* B, int ldb, int M, int N, int K, void* C, int ldc,
                           int c_fp32, const float* bias, int act, void* Z) {
    // one error word per device, allocated on first use
    static std::mutex mu;
    static int* d_err[64] = {nullptr};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return WP_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!d_err[dev] && cudaMalloc(&d_err[dev], sizeof(int)) != cudaSuccess) return WP_ERR_OOM;
    }
    cudaMemsetAsync(d_err[dev], 0, sizeof(int), 0);
    cudaError_t e = wp_gemm_bf16_tn(A, lda, B, ldb, M, N, K, C, ldc, c_fp32, bias, act, Z, 0, d_err[dev], 0);
    if (e == cudaErrorInvalidValue) return WP_ERR_INVALID;
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, d_err[dev], sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return WP_ERR_CUDA;
    return err ? WP_ERR_TIMEOUT : WP_OK;
}

wp_status wp_hmm_count_flops(wp_ctx* ctx, const double* rads, int R, double dist_cutoff, double* out_flops) {
    if (!ctx || R < 0 || !out_flops || (R > 0 && !rads)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    *out_flops = 0.0;
    if (R == 0 || ctx->P == 0) return WP_OK;
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    WP_CUDA(ctx->d_flops.ensure(sizeof(double) * R), "alloc flops");
    WP_CUDA(cudaMemsetAsync(ctx->d_flops.p, 0, sizeof(double) * R, ctx->stream), "clear flops");
    st = run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, nullptr, nullptr, MODE_FLOPS, nullptr,
                   nullptr, nullptr, nullptr, nullptr, ctx->d_flops.as<double>());
    if (st != WP_OK) return st;
    std::vector<double> per(R);
    WP_CUDA(cudaMemcpyAsync(per.data(), ctx->d_flops.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy flops");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    double s = 0.0;
    for (double v : per) s += v;
    *out_flops = s;
    return WP_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ learned proposal
struct wp_mlp {
    int device = 0;
    int P = 0, Ppad = 0, H = 0, TC = 0;
    int cap = 0;              // batch capacity of the activation buffers
    long long steps = 0;      // Adam steps taken
    // FP32: W1 b1 W2 b2 W3 b3, each with grad, Adam m, v
    DevBuf w[6], g[6], m[6], v[6];
    long n[6] = {0, 0, 0, 0, 0, 0};
    DevBuf W1b, W2b, W3b, W2T, W3T;  // BF16 copies
    DevBuf X, XT, Z1, H1, H1T, Z2, H2, H2T, dL, dLT, dZ2, dZ2T, dZ1, dZ1T, L, dH2, dH1, loss, labels, xsim, err;
    DevBuf topi, topp, mass, counts, loss_sum, tkfail;
};

namespace {

typedef __nv_bfloat16 bf16;

#define MLP_CUDA(call, what)                                    \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what); \
    } while (0)

wp_status mlp_gemm(wp_ctx* ctx, wp_mlp* m, const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                   void* C, int ldc, int c_fp32, const float* bias, int act, void* Z) {
    cudaError_t e = wp_gemm_bf16_tn(A, lda, B, ldb, M, N, K, C, ldc, c_fp32, bias, act, Z, 0, m->err.as<int>(),
                                    ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "tensor-core GEMM launch");
    return WP_OK;
}

wp_status mlp_ensure(wp_ctx* ctx, wp_mlp* m, int B) {
    if (B <= m->cap) return WP_OK;
    const size_t b = (size_t)B, H = m->H, Pp = m->Ppad;
    MLP_CUDA(m->X.ensure(sizeof(bf16) * b * 64), "alloc");
    MLP_CUDA(m->XT.ensure(sizeof(bf16) * b * 64), "alloc");
    for (DevBuf* d : {&m->Z1, &m->H1, &m->H1T, &m->Z2, &m->H2, &m->H2T, &m->dZ2, &m->dZ2T, &m->dZ1, &m->dZ1T})
        MLP_CUDA(d->ensure(sizeof(bf16) * b * H), "alloc activations");
    MLP_CUDA(m->dL.ensure(sizeof(bf16) * b * Pp), "alloc logits gradient");
    MLP_CUDA(m->dLT.ensure(sizeof(bf16) * b * Pp), "alloc logits gradient");
    MLP_CUDA(m->L.ensure(sizeof(float) * b * Pp), "alloc logits");
    MLP_CUDA(m->dH2.ensure(sizeof(float) * b * H), "alloc");
    MLP_CUDA(m->dH1.ensure(sizeof(float) * b * H), "alloc");
    MLP_CUDA(m->loss.ensure(sizeof(double) * b), "alloc");
    MLP_CUDA(m->labels.ensure(sizeof(int) * b), "alloc");
    MLP_CUDA(m->xsim.ensure(sizeof(float) * b * m->TC), "alloc");
    m->cap = B;
    return WP_OK;
}

// BF16 copies (and transposes) of the master weights.
wp_status mlp_refresh(wp_ctx* ctx, wp_mlp* m) {
    MLP_CUDA(wp_mlp_launch_to_bf16(m->w[0].as<float>(), m->n[0], m->W1b.as<bf16>(), ctx->stream), "bf16");
    MLP_CUDA(wp_mlp_launch_to_bf16(m->w[2].as<float>(), m->n[2], m->W2b.as<bf16>(), ctx->stream), "bf16");
    MLP_CUDA(wp_mlp_launch_to_bf16(m->w[4].as<float>(), m->n[4], m->W3b.as<bf16>(), ctx->stream), "bf16");
    MLP_CUDA(wp_mlp_launch_transpose(m->W2b.as<bf16>(), m->H, m->H, m->H, m->W2T.as<bf16>(), m->H, ctx->stream), "T");
    MLP_CUDA(wp_mlp_launch_transpose(m->W3b.as<bf16>(), m->Ppad, m->H, m->H, m->W3T.as<bf16>(), m->Ppad, ctx->stream),
             "T");
    ctx->launches += 5;
    return WP_OK;
}

// Logits of B inputs already in m->X.
wp_status mlp_forward(wp_ctx* ctx, wp_mlp* m, int B) {
    const int H = m->H, Pp = m->Ppad;
    wp_status st = mlp_gemm(ctx, m, m->X.p, 64, m->W1b.p, 64, B, H, 64, m->H1.p, H, 0, m->w[1].as<float>(), 1, m->Z1.p);
    if (st != WP_OK) return st;
    st = mlp_gemm(ctx, m, m->H1.p, H, m->W2b.p, H, B, H, H, m->H2.p, H, 0, m->w[3].as<float>(), 1, m->Z2.p);
    if (st != WP_OK) return st;
    return mlp_gemm(ctx, m, m->H2.p, H, m->W3b.p, H, B, Pp, H, m->L.p, Pp, 1, m->w[5].as<float>(), 0, nullptr);
}

// One optimiser step on B inputs in m->X with labels in m->labels (lr 0:
// gradients only).
wp_status mlp_step(wp_ctx* ctx, wp_mlp* m, int B, float lr) {
    const int H = m->H, Pp = m->Ppad;
    cudaStream_t s = ctx->stream;
    wp_status st = mlp_forward(ctx, m, B);
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_softmax_ce(m->L.as<float>(), B, m->P, Pp, m->labels.as<int>(), 1.0f / (float)B,
                                      m->dL.as<bf16>(), m->loss.as<double>(), s), "softmax");
    MLP_CUDA(wp_mlp_launch_transpose(m->dL.as<bf16>(), B, Pp, Pp, m->dLT.as<bf16>(), B, s), "T");
    MLP_CUDA(wp_mlp_launch_transpose(m->H2.as<bf16>(), B, H, H, m->H2T.as<bf16>(), B, s), "T");
    ctx->launches += 3;
    st = mlp_gemm(ctx, m, m->dLT.p, B, m->H2T.p, B, Pp, H, B, m->g[4].p, H, 1, nullptr, 0, nullptr);  // dW3
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_colsum(m->dL.as<bf16>(), B, Pp, Pp, m->g[5].as<float>(), s), "colsum");
    st = mlp_gemm(ctx, m, m->dL.p, Pp, m->W3T.p, Pp, B, H, Pp, m->dH2.p, H, 1, nullptr, 0, nullptr);  // dH2
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_gelu_bwd(m->dH2.as<float>(), m->Z2.as<bf16>(), (long)B * H, m->dZ2.as<bf16>(), s), "gelu'");
    MLP_CUDA(wp_mlp_launch_transpose(m->dZ2.as<bf16>(), B, H, H, m->dZ2T.as<bf16>(), B, s), "T");
    MLP_CUDA(wp_mlp_launch_transpose(m->H1.as<bf16>(), B, H, H, m->H1T.as<bf16>(), B, s), "T");
    ctx->launches += 4;
    st = mlp_gemm(ctx, m, m->dZ2T.p, B, m->H1T.p, B, H, H, B, m->g[2].p, H, 1, nullptr, 0, nullptr);  // dW2
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_colsum(m->dZ2.as<bf16>(), B, H, H, m->g[3].as<float>(), s), "colsum");
    st = mlp_gemm(ctx, m, m->dZ2.p, H, m->W2T.p, H, B, H, H, m->dH1.p, H, 1, nullptr, 0, nullptr);  // dH1
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_gelu_bwd(m->dH1.as<float>(), m->Z1.as<bf16>(), (long)B * H, m->dZ1.as<bf16>(), s), "gelu'");
    MLP_CUDA(wp_mlp_launch_transpose(m->dZ1.as<bf16>(), B, H, H, m->dZ1T.as<bf16>(), B, s), "T");
    MLP_CUDA(wp_mlp_launch_transpose(m->X.as<bf16>(), B, 64, 64, m->XT.as<bf16>(), B, s), "T");
    ctx->launches += 4;
    st = mlp_gemm(ctx, m, m->dZ1T.p, B, m->XT.p, B, H, 64, B, m->g[0].p, 64, 1, nullptr, 0, nullptr);  // dW1
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_colsum(m->dZ1.as<bf16>(), B, H, H, m->g[1].as<float>(), s), "colsum");
    ctx->launches++;
    if (lr > 0.0f) {
        m->steps++;
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        const float bc1 = 1.0f - powf(b1, (float)m->steps), bc2 = 1.0f - powf(b2, (float)m->steps);
        bf16* wb[6] = {m->W1b.as<bf16>(), nullptr, m->W2b.as<bf16>(), nullptr, m->W3b.as<bf16>(), nullptr};
        for (int i = 0; i < 6; i++) {
            MLP_CUDA(wp_mlp_launch_adam(m->w[i].as<float>(), m->g[i].as<float>(), m->m[i].as<float>(),
                                        m->v[i].as<float>(), m->n[i], lr, b1, b2, eps, bc1, bc2, wb[i], s), "adam");
            ctx->launches++;
        }
        MLP_CUDA(wp_mlp_launch_transpose(m->W2b.as<bf16>(), H, H, H, m->W2T.as<bf16>(), H, s), "T");
        MLP_CUDA(wp_mlp_launch_transpose(m->W3b.as<bf16>(), Pp, H, H, m->W3T.as<bf16>(), Pp, s), "T");
        ctx->launches += 2;
    }
    return WP_OK;
}

wp_status mlp_check(wp_ctx* ctx, wp_mlp* m) {
    if (!m) return WP_ERR_INVALID;
    if (!ctx->have_model || !ctx->have_peps) return fail(ctx, WP_ERR_STATE, "model or peptides not uploaded");
    if (ctx->P != m->P || ctx->hm.T * ctx->hm.C != m->TC)
        return fail(ctx, WP_ERR_STATE, "the network was built for another peptide set or read shape");
    return WP_OK;
}

wp_status mlp_finish(wp_ctx* ctx, wp_mlp* m) {
    MLP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    int err = 0;
    MLP_CUDA(cudaMemcpy(&err, m->err.p, sizeof(int), cudaMemcpyDeviceToHost), "read err");
    if (err) return fail(ctx, WP_ERR_TIMEOUT, "a tensor-core GEMM pipeline wait expired");
    return WP_OK;
}

// Top-h proposals for R reads on the device (FP64 [R][TC]), in chunks of
// the batch capacity: ascending peptide indices by logit in d_idx [R][h],
// probabilities in d_prob, candidate mass (sum prob x count) in d_mass.
wp_status mlp_propose_dev(wp_ctx* ctx, wp_mlp* m, const double* d_rads, int R, int h, int* d_idx, float* d_prob,
                          double* d_mass) {
    const int chunk = 8192;
    wp_status st = mlp_ensure(ctx, m, chunk);
    if (st != WP_OK) return st;
    MLP_CUDA(m->counts.ensure(sizeof(int) * std::max(ctx->P, 1)), "alloc");
    MLP_CUDA(cudaMemcpyAsync(m->counts.p, ctx->counts.data(), sizeof(int) * ctx->P, cudaMemcpyHostToDevice,
                             ctx->stream), "copy");
    for (int r0 = 0; r0 < R; r0 += chunk) {
        const int n = std::min(chunk, R - r0);
        MLP_CUDA(wp_mlp_launch_input(nullptr, d_rads + (size_t)r0 * m->TC, n, m->TC, m->X.as<bf16>(), ctx->stream),
                 "input");
        ctx->launches++;
        {
            TimedLaunch tl(ctx, 4);
            st = mlp_forward(ctx, m, n);
            if (st != WP_OK) return st;
        }
        TimedLaunch tl(ctx, 5);
        MLP_CUDA(m->tkfail.ensure(sizeof(int) * ((size_t)chunk + 1)), "alloc top-k scratch");
        MLP_CUDA(wp_mlp_launch_topk(m->L.as<float>(), n, m->P, m->Ppad, h, m->counts.as<int>(), d_idx + (size_t)r0 * h,
                                    d_prob + (size_t)r0 * h, d_mass + r0, m->tkfail.as<int>(), ctx->stream),
                 "top-k");
        ctx->launches++;
    }
    return WP_OK;
}

}  // namespace

extern "C" {

wp_status wp_mlp_create(wp_ctx* ctx, int hidden, unsigned long long seed, wp_mlp** out) {
    if (!ctx || !out || hidden < 64 || hidden % 64) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!ctx->have_model || !ctx->have_peps) return fail(ctx, WP_ERR_STATE, "model or peptides not uploaded");
    if (ctx->P < 1) return fail(ctx, WP_ERR_INVALID, "no peptides");
    const int TC = ctx->hm.T * ctx->hm.C;
    if (TC > 64) return fail(ctx, WP_ERR_UNSUPPORTED, "the network takes timesteps x channels <= 64");
    wp_mlp* m = new wp_mlp();
    m->device = ctx->device;
    m->P = ctx->P;
    m->Ppad = (ctx->P + 63) / 64 * 64;
    m->H = hidden;
    m->TC = TC;
    const long H = hidden, Pp = m->Ppad;
    const long sizes[6] = {H * 64, H, H * H, H, Pp * H, Pp};
    for (int i = 0; i < 6; i++) {
        m->n[i] = sizes[i];
        for (DevBuf* d : {&m->w[i], &m->g[i], &m->m[i], &m->v[i]}) {
            if (d->ensure(sizeof(float) * sizes[i]) != cudaSuccess) {
                delete m;
                return fail(ctx, WP_ERR_OOM, "alloc network");
            }
            cudaMemsetAsync(d->p, 0, sizeof(float) * sizes[i], ctx->stream);
        }
    }
    if (m->W1b.ensure(sizeof(bf16) * H * 64) || m->W2b.ensure(sizeof(bf16) * H * H) ||
        m->W3b.ensure(sizeof(bf16) * Pp * H) || m->W2T.ensure(sizeof(bf16) * H * H) ||
        m->W3T.ensure(sizeof(bf16) * Pp * H) || m->err.ensure(sizeof(int)) || m->loss_sum.ensure(sizeof(double))) {
        delete m;
        return fail(ctx, WP_ERR_OOM, "alloc network");
    }
    cudaMemsetAsync(m->err.p, 0, sizeof(int), ctx->stream);
    // He-style initialisation: N(0, 2 / fan_in) for the GELU layers,
    // N(0, 1 / fan_in) for the logits; biases zero; padded classes zero.
    cudaError_t e = wp_mlp_launch_init(m->w[0].as<float>(), H, 64, H, sqrtf(2.0f / (float)TC), seed, ctx->stream);
    if (e == cudaSuccess) e = wp_mlp_launch_init(m->w[2].as<float>(), H, H, H, sqrtf(2.0f / (float)H), seed + 1, ctx->stream);
    if (e == cudaSuccess) e = wp_mlp_launch_init(m->w[4].as<float>(), Pp, H, m->P, sqrtf(1.0f / (float)H), seed + 2, ctx->stream);
    ctx->launches += 3;
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(ctx, e, "init network");
    }
    wp_status st = mlp_refresh(ctx, m);
    if (st == WP_OK) st = mlp_finish(ctx, m);
    if (st != WP_OK) {
        delete m;
        return st;
    }
    *out = m;
    return WP_OK;
}

void wp_mlp_destroy(wp_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    delete m;
}

wp_status wp_mlp_train(wp_ctx* ctx, wp_mlp* m, long long num_reads, int batch, float lr, unsigned long long seed,
                       double* out_mean_loss) {
    if (!ctx || !m || num_reads < 0 || batch < 64 || batch % 64 || !(lr >= 0.0f)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    st = mlp_ensure(ctx, m, batch);
    if (st != WP_OK) return st;
    const long long steps = (num_reads + batch - 1) / batch;
    std::vector<double> hl(batch);
    double loss_sum = 0.0;
    long long counted = 0;
    for (long long k = 0; k < steps; k++) {
        // fresh reads for every step: subsequence streams of seed + k
        st = sim_device(ctx, batch, seed + (unsigned long long)k * 0x9E3779B97F4A7C15ull, m->xsim.as<float>(),
                        nullptr, m->labels.as<int>(), nullptr);
        if (st != WP_OK) return st;
        MLP_CUDA(wp_mlp_launch_input(m->xsim.as<float>(), nullptr, batch, m->TC, m->X.as<bf16>(), ctx->stream), "input");
        ctx->launches++;
        {
            TimedLaunch tl(ctx, 0);
            st = mlp_step(ctx, m, batch, lr);
            if (st != WP_OK) return st;
        }
        if (out_mean_loss && (k + 1 == steps || (k & 63) == 0)) {
            // sample the loss every 64 steps and at the end
            MLP_CUDA(cudaMemcpyAsync(hl.data(), m->loss.p, sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->stream),
                     "copy loss");
            MLP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
            double sl = 0.0;
            for (double x : hl) sl += x;
            loss_sum = sl / batch;
            counted++;
        }
    }
    st = mlp_finish(ctx, m);
    if (st != WP_OK) return st;
    if (out_mean_loss) *out_mean_loss = counted ? loss_sum : 0.0;
    return WP_OK;
}

wp_status wp_mlp_train_step(wp_ctx* ctx, wp_mlp* m, const float* d_x, const int32_t* d_labels, int B, float lr,
                            double* out_loss) {
    if (!ctx || !m || !d_x || !d_labels || B < 64 || B % 64 || !(lr >= 0.0f)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    st = mlp_ensure(ctx, m, B);
    if (st != WP_OK) return st;
    MLP_CUDA(wp_mlp_launch_input(d_x, nullptr, B, m->TC, m->X.as<bf16>(), ctx->stream), "input");
    MLP_CUDA(cudaMemcpyAsync(m->labels.p, d_labels, sizeof(int) * B, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    ctx->launches++;
    st = mlp_step(ctx, m, B, lr);
    if (st != WP_OK) return st;
    st = mlp_finish(ctx, m);
    if (st != WP_OK) return st;
    if (out_loss) {
        std::vector<double> hl(B);
        MLP_CUDA(cudaMemcpy(hl.data(), m->loss.p, sizeof(double) * B, cudaMemcpyDeviceToHost), "copy loss");
        double sl = 0.0;
        for (double x : hl) sl += x;
        *out_loss = sl / B;
    }
    return WP_OK;
}

wp_status wp_mlp_get(wp_mlp* m, int which, int grad, float* out) {
    if (!m || which < 0 || which > 5 || !out) return WP_ERR_INVALID;
    cudaSetDevice(m->device);
    DevBuf& b = grad ? m->g[which] : m->w[which];
    if (cudaMemcpy(out, b.p, sizeof(float) * m->n[which], cudaMemcpyDeviceToHost) != cudaSuccess) return WP_ERR_CUDA;
    return WP_OK;
}

wp_status wp_mlp_set(wp_ctx* ctx, wp_mlp* m, int which, const float* in) {
    if (!ctx || !m || which < 0 || which > 5 || !in) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    MLP_CUDA(cudaMemcpyAsync(m->w[which].p, in, sizeof(float) * m->n[which], cudaMemcpyHostToDevice, ctx->stream),
             "copy");
    wp_status st = mlp_refresh(ctx, m);
    if (st != WP_OK) return st;
    return mlp_finish(ctx, m);
}

wp_status wp_mlp_shape(const wp_mlp* m, int which, long long* rows, long long* cols) {
    if (!m || which < 0 || which > 5) return WP_ERR_INVALID;
    const long long r[6] = {m->H, m->H, m->H, m->H, m->Ppad, m->Ppad};
    const long long c[6] = {64, 1, m->H, 1, m->H, 1};
    if (rows) *rows = r[which];
    if (cols) *cols = c[which];
    return WP_OK;
}

wp_status wp_mlp_logits(wp_ctx* ctx, wp_mlp* m, const double* rads, int R, float* out) {
    if (!ctx || !m || R < 0 || (R > 0 && (!rads || !out))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    const int chunk = 8192;
    st = mlp_ensure(ctx, m, chunk);
    if (st != WP_OK) return st;
    for (int r0 = 0; r0 < R; r0 += chunk) {
        const int n = std::min(chunk, R - r0);
        MLP_CUDA(wp_mlp_launch_input(nullptr, ctx->d_rads.as<double>() + (size_t)r0 * m->TC, n, m->TC, m->X.as<bf16>(),
                                     ctx->stream), "input");
        st = mlp_forward(ctx, m, n);
        if (st != WP_OK) return st;
        MLP_CUDA(cudaMemcpy2DAsync(out + (size_t)r0 * m->P, sizeof(float) * m->P, m->L.p, sizeof(float) * m->Ppad,
                                   sizeof(float) * m->P, n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    }
    return mlp_finish(ctx, m);
}

wp_status wp_mlp_propose(wp_ctx* ctx, wp_mlp* m, const double* rads, int R, int h, int32_t* out_idx, float* out_prob,
                         double* out_mass) {
    if (!ctx || !m || R < 0 || h < 1 || h > 1024 || (R > 0 && (!rads || !out_idx || !out_prob))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    if (h > m->P) return fail(ctx, WP_ERR_INVALID, "h exceeds the number of peptides");
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    MLP_CUDA(ctx->d_nn_cand_pep.ensure(sizeof(int) * (size_t)R * h), "alloc");
    MLP_CUDA(ctx->d_nn_cand_score.ensure(sizeof(float) * (size_t)R * h), "alloc");
    MLP_CUDA(ctx->d_nn_subfrac.ensure(sizeof(double) * R), "alloc");
    st = mlp_propose_dev(ctx, m, ctx->d_rads.as<double>(), R, h, ctx->d_nn_cand_pep.as<int>(),
                         reinterpret_cast<float*>(ctx->d_nn_cand_score.p), ctx->d_nn_subfrac.as<double>());
    if (st != WP_OK) return st;
    MLP_CUDA(cudaMemcpyAsync(out_idx, ctx->d_nn_cand_pep.p, sizeof(int) * (size_t)R * h, cudaMemcpyDeviceToHost,
                             ctx->stream), "copy");
    MLP_CUDA(cudaMemcpyAsync(out_prob, ctx->d_nn_cand_score.p, sizeof(float) * (size_t)R * h, cudaMemcpyDeviceToHost,
                             ctx->stream), "copy");
    if (out_mass)
        MLP_CUDA(cudaMemcpyAsync(out_mass, ctx->d_nn_subfrac.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream),
                 "copy");
    return mlp_finish(ctx, m);
}

static wp_status mlp_hybrid_run(wp_ctx* ctx, wp_mlp* m, const double* d_rads, int R, int h, double dist_cutoff,
                                int* d_id, double* d_score, double* d_total) {
    MLP_CUDA(ctx->d_nn_cand_pep.ensure(sizeof(int) * (size_t)R * h), "alloc");
    MLP_CUDA(ctx->d_nn_cand_score.ensure(sizeof(float) * (size_t)R * h), "alloc");
    MLP_CUDA(ctx->d_nn_subfrac.ensure(sizeof(double) * R), "alloc");
    MLP_CUDA(ctx->d_nn_ncand.ensure(sizeof(int) * R), "alloc");
    wp_status st = mlp_propose_dev(ctx, m, d_rads, R, h, ctx->d_nn_cand_pep.as<int>(),
                                   reinterpret_cast<float*>(ctx->d_nn_cand_score.p), ctx->d_nn_subfrac.as<double>());
    if (st != WP_OK) return st;
    // every read has h candidates: [R][h] is already the ragged layout
    std::vector<int> off(R + 1), nc(R, h);
    for (int r = 0; r <= R; r++) off[r] = r * h;
    MLP_CUDA(ctx->d_nn_cand_off.ensure(sizeof(int) * (R + 1)), "alloc");
    MLP_CUDA(cudaMemcpyAsync(ctx->d_nn_cand_off.p, off.data(), sizeof(int) * (R + 1), cudaMemcpyHostToDevice,
                             ctx->stream), "copy");
    MLP_CUDA(cudaMemcpyAsync(ctx->d_nn_ncand.p, nc.data(), sizeof(int) * R, cudaMemcpyHostToDevice, ctx->stream), "copy");
    st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, off.data(), MODE_CLASSIFY, nullptr, d_id, d_score, d_total,
                   nullptr, nullptr, ctx->d_nn_cand_pep.as<int>(), ctx->d_nn_cand_off.as<int>());
    if (st != WP_OK) return st;
    MLP_CUDA(wp_launch_hybrid_finish(ctx->d_nn_ncand.as<int>(), ctx->d_nn_subfrac.as<double>(), R, d_id, d_score,
                                     d_total, ctx->stream), "finish");
    ctx->launches++;
    return WP_OK;
}

wp_status wp_mlp_hybrid_classify(wp_ctx* ctx, wp_mlp* m, const double* rads, int R, int h, double dist_cutoff,
                                 int32_t* out_id, double* out_score, double* out_total) {
    if (!ctx || !m || R < 0 || h < 1 || h > 1024 || (R > 0 && (!rads || !out_id || !out_score || !out_total)))
        return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    if (h > m->P) return fail(ctx, WP_ERR_INVALID, "h exceeds the number of peptides");
    st = upload_reads(ctx, rads, R);
    if (st != WP_OK) return st;
    MLP_CUDA(ctx->d_out_id.ensure(sizeof(int) * R), "alloc");
    MLP_CUDA(ctx->d_out_score.ensure(sizeof(double) * R), "alloc");
    MLP_CUDA(ctx->d_out_total.ensure(sizeof(double) * R), "alloc");
    st = mlp_hybrid_run(ctx, m, ctx->d_rads.as<double>(), R, h, dist_cutoff, ctx->d_out_id.as<int>(),
                        ctx->d_out_score.as<double>(), ctx->d_out_total.as<double>());
    if (st != WP_OK) return st;
    MLP_CUDA(cudaMemcpyAsync(out_id, ctx->d_out_id.p, sizeof(int) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    MLP_CUDA(cudaMemcpyAsync(out_score, ctx->d_out_score.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    MLP_CUDA(cudaMemcpyAsync(out_total, ctx->d_out_total.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy");
    st = finish(ctx);
    if (st != WP_OK) return st;
    return mlp_finish(ctx, m);
}

wp_status wp_mlp_hybrid_classify_device(wp_ctx* ctx, wp_mlp* m, const double* d_rads, int R, int h,
                                        double dist_cutoff, int32_t* d_id, double* d_score, double* d_total) {
    if (!ctx || !m || R < 0 || h < 1 || h > 1024 || (R > 0 && (!d_rads || !d_id || !d_score || !d_total)))
        return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = mlp_check(ctx, m);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    if (h > m->P) return fail(ctx, WP_ERR_INVALID, "h exceeds the number of peptides");
    st = mlp_hybrid_run(ctx, m, d_rads, R, h, dist_cutoff, d_id, d_score, d_total);
    if (st != WP_OK) return st;
    st = finish(ctx);
    if (st != WP_OK) return st;
    return mlp_finish(ctx, m);
}

}  // extern "C"
