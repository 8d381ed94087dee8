// wp_capi.cu -- host side of the C ABI declared in include/whatprot_gb300.h.
//
// The context owns one CUDA stream and the device copies of the model
// (DevModel) and peptide set (PeptideRec[]).  A classify call:
//   1. copies the reads to the device (or takes device pointers),
//   2. runs the prep kernel (per-read emission boxes and factors),
//   3. runs the forward kernel once per shape bucket -- peptides are bucketed
//      by the size of their Edman slice S = prod_c (D_c + 1) so that each
//      launch sizes its per-warp shared-memory buffers to its bucket --
//      with one CTA per (read, chunk of the bucket's peptides),
//   4. combines the per-chunk partials per read and copies the results back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wp_common.cuh"

// Kernels (wp_kernels.cu).
__global__ void wp_prep_reads_kernel(const DevModel*, const double*, int, unsigned, double,
                                     uint8_t*, uint8_t*, EmitEntry*, int);
__global__ void wp_combine_kernel(int, const int*, const int*, const int*, const float*,
                                  const int*, const double*, const int*, int32_t*, double*,
                                  double*, double*);
__global__ void wp_count_flops_kernel(const DevModel*, const PeptideRec*, int, const uint8_t*,
                                      const uint8_t*, int, double*);
size_t wp_forward_smem_bytes(int T, int S_cap, int C, bool has_block, int warps);
cudaError_t wp_launch_fma_probe(int blocks, int threads, int iters, cudaStream_t stream, float* sink);
cudaError_t wp_launch_forward(bool has_block, int grid, int threads, size_t smem,
                              cudaStream_t stream, const TileArgs& args);

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
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

struct Bucket {
    int S_cap;
    std::vector<int> peps;  // ascending peptide indices
};

}  // namespace

struct wp_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string err;
    long long launches = 0;
    int smem_optin = 0;

    bool have_model = false;
    DevModel hm;
    DevBuf d_model;

    bool have_peps = false;
    std::vector<int16_t> seqs;
    std::vector<int32_t> offsets, ids, counts;
    int P = 0;
    // Derived at plan time (need C and T).
    int plan_C = -1, plan_T = -1;
    int dmax = 0;
    std::vector<PeptideRec> recs;
    std::vector<Bucket> buckets;
    DevBuf d_peps, d_ids, d_counts, d_list, d_chunk_b, d_chunk_e;
    std::vector<int> list;  // concatenated bucket lists
    std::vector<int> list_off;  // per bucket start in list

    // Kernel timing.
    bool timing = false;
    struct Timed {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;
    double t_ms[4] = {0, 0, 0, 0};
    long long t_n[4] = {0, 0, 0, 0};

    // Per-call scratch.
    DevBuf d_rads, d_lo, d_hi, d_table, d_part_key, d_part_pep, d_part_mant, d_part_expo,
            d_part_total, d_read_tile_off, d_out_id, d_out_score, d_out_total, d_out_log,
            d_logp, d_flops, d_err, d_tiles, d_cand_list, d_cand_key;
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

#define WP_CUDA(call, what)                                   \
    do {                                                      \
        cudaError_t _e = (call);                              \
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
void binomial_table(double q, int max_n, float* out) {
    std::vector<double> tab((max_n + 1) * (max_n + 2) / 2);
    double p = 1.0 - q;
    tab[0] = 1.0;
    for (int i = 1; i <= max_n; i++) {
        tab[i * (i + 1) / 2] = tab[(i - 1) * i / 2] * q;
        for (int j = 1; j < i; j++)
            tab[i * (i + 1) / 2 + j] = tab[(i - 1) * i / 2 + j] * q + tab[(i - 1) * i / 2 + j - 1] * p;
        tab[i * (i + 1) / 2 + i] = tab[(i - 1) * i / 2 + i - 1] * p;
    }
    for (size_t k = 0; k < tab.size(); k++) out[k] = (float)tab[k];
}

// Build per-peptide records and shape buckets for (C, T).
wp_status plan_peptides(wp_ctx* ctx) {
    const int C = ctx->hm.C, T = ctx->hm.T;
    if (ctx->plan_C == C && ctx->plan_T == T) return WP_OK;
    const int P = ctx->P;
    ctx->recs.assign(P, PeptideRec());
    ctx->dmax = 0;
    std::vector<int> S(P);
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
        int prod = 1;
        for (int c = 0; c < C; c++) {
            if (cnt[c] > WP_MAX_DYES_PER_CHANNEL)
                return fail(ctx, WP_ERR_UNSUPPORTED, "dye-seq " + std::to_string(i) +
                                                             " has more than 15 dyes on one channel");
            rec.D[c] = (uint8_t)cnt[c];
            ctx->dmax = std::max(ctx->dmax, cnt[c]);
            prod *= cnt[c] + 1;
        }
        S[i] = prod;
        // DyeTrack(e, c) for c = dye_seq[e] (common/dye-track.cc:26-43).
        int rem[WP_MAX_CHANNELS];
        memcpy(rem, cnt, sizeof(rem));
        for (int e = 0; e < WP_MAX_TIMESTEPS; e++) {
            int d = e < len ? s[e] : -1;
            rec.dye[e] = (int8_t)d;
            rec.tot[e] = (uint8_t)(d >= 0 ? rem[d] : 0);
            if (d >= 0) rem[d]--;
        }
    }
    // Buckets by S (powers of two from 16).
    ctx->buckets.clear();
    int max_S = 1;
    for (int i = 0; i < P; i++) max_S = std::max(max_S, S[i]);
    for (int cap = 16;; cap *= 2) {
        Bucket b;
        b.S_cap = cap;
        int lo = cap == 16 ? 0 : cap / 2;
        for (int i = 0; i < P; i++)
            if (S[i] > lo && S[i] <= cap) b.peps.push_back(i);
        if (!b.peps.empty()) ctx->buckets.push_back(b);
        if (cap >= max_S) break;
    }
    ctx->list.clear();
    ctx->list_off.clear();
    for (auto& b : ctx->buckets) {
        ctx->list_off.push_back((int)ctx->list.size());
        ctx->list.insert(ctx->list.end(), b.peps.begin(), b.peps.end());
    }
    ctx->list_off.push_back((int)ctx->list.size());
    WP_CUDA(ctx->d_peps.ensure(sizeof(PeptideRec) * std::max(P, 1)), "alloc peptides");
    WP_CUDA(cudaMemcpyAsync(ctx->d_peps.p, ctx->recs.data(), sizeof(PeptideRec) * P,
                            cudaMemcpyHostToDevice, ctx->stream), "copy peptides");
    WP_CUDA(ctx->d_list.ensure(sizeof(int) * std::max<size_t>(ctx->list.size(), 1)), "alloc list");
    WP_CUDA(cudaMemcpyAsync(ctx->d_list.p, ctx->list.data(), sizeof(int) * ctx->list.size(),
                            cudaMemcpyHostToDevice, ctx->stream), "copy list");
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

int warps_for(wp_ctx* ctx, int S_cap) {
    const int T = ctx->hm.T, C = ctx->hm.C;
    bool hb = ctx->hm.has_block != 0;
    for (int w = 16; w >= 1; w--)
        if (wp_forward_smem_bytes(T, S_cap, C, hb, w) <= (size_t)ctx->smem_optin) return w;
    return 0;
}

constexpr int kChunk = 256;  // peptides per CTA in the all-peptides mode



// Run prep + forward (+ combine when outputs given) on device-resident reads.
wp_status run_batch(wp_ctx* ctx, const double* d_rads, int R, double dist_cutoff,
                    const int32_t* h_cand, const int32_t* h_cand_off, double* d_logp,
                    int32_t* d_out_id, double* d_out_score, double* d_out_total, double* d_out_log) {
    const int C = ctx->hm.C, T = ctx->hm.T;
    wp_status st = plan_peptides(ctx);
    if (st != WP_OK) return st;
    const int W = ctx->dmax + 1;
    const int entries = wp_read_table_entries(T, C, W, ctx->hm.interacting);
    WP_CUDA(ctx->d_lo.ensure((size_t)R * T * C), "alloc boxes");
    WP_CUDA(ctx->d_hi.ensure((size_t)R * T * C), "alloc boxes");
    WP_CUDA(ctx->d_table.ensure(sizeof(EmitEntry) * (size_t)R * entries), "alloc emission table");
    WP_CUDA(ctx->d_err.ensure(sizeof(int)), "alloc err");
    WP_CUDA(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(int), ctx->stream), "clear err");
    {
        long n = (long)R * T;
        int threads = 128;
        int blocks = (int)((n + threads - 1) / threads);
        if (blocks > 0) {
            TimedLaunch tl(ctx, 1);
            wp_prep_reads_kernel<<<blocks, threads, 0, ctx->stream>>>(
                    ctx->d_model.as<DevModel>(), d_rads, R, (unsigned)ctx->dmax, dist_cutoff,
                    ctx->d_lo.as<uint8_t>(), ctx->d_hi.as<uint8_t>(), ctx->d_table.as<EmitEntry>(),
                    entries);
            ctx->launches++;
            WP_CUDA(cudaGetLastError(), "prep launch");
        }
    }
    const bool classify = d_out_id != nullptr;
    TileArgs a;
    memset(&a, 0, sizeof(a));
    a.model = ctx->d_model.as<DevModel>();
    a.peps = ctx->d_peps.as<PeptideRec>();
    a.box_lo = ctx->d_lo.as<uint8_t>();
    a.box_hi = ctx->d_hi.as<uint8_t>();
    a.table = ctx->d_table.as<EmitEntry>();
    a.entries = entries;
    a.W = W;
    a.num_peptides = ctx->P;
    a.counts = ctx->d_counts.as<int>();
    a.out_logp = d_logp;
    a.err = ctx->d_err.as<int>();
    const bool hb = ctx->hm.has_block != 0;

    // Tiles: (read, bucket, chunk).  In candidate mode each read's candidates
    // are bucketed on the host.
    std::vector<int> tile_read, tile_begin, tile_end, tile_bucket, read_tile_off(R + 1, 0);
    std::vector<int> cand_list, cand_key;
    if (h_cand) {
        std::vector<int> bucket_of(ctx->P, -1);
        for (size_t b = 0; b < ctx->buckets.size(); b++)
            for (int p : ctx->buckets[b].peps) bucket_of[p] = (int)b;
        std::vector<std::vector<std::pair<int, int>>> per(ctx->buckets.size());
        for (int r = 0; r < R; r++) {
            for (auto& v : per) v.clear();
            for (int k = h_cand_off[r]; k < h_cand_off[r + 1]; k++) {
                int p = h_cand[k];
                if (p < 0 || p >= ctx->P) return fail(ctx, WP_ERR_INVALID, "candidate index out of range");
                per[bucket_of[p]].push_back({p, k - h_cand_off[r]});
            }
            for (size_t b = 0; b < per.size(); b++) {
                for (size_t s0 = 0; s0 < per[b].size(); s0 += kChunk) {
                    size_t s1 = std::min(per[b].size(), s0 + kChunk);
                    tile_read.push_back(r);
                    tile_begin.push_back((int)cand_list.size());
                    for (size_t q = s0; q < s1; q++) {
                        cand_list.push_back(per[b][q].first);
                        cand_key.push_back(per[b][q].second);
                    }
                    tile_end.push_back((int)cand_list.size());
                    tile_bucket.push_back((int)b);
                }
            }
            read_tile_off[r + 1] = (int)tile_read.size();
        }
    } else {
        int per_read = 0;
        std::vector<int> cb, ce, cbk;
        for (size_t b = 0; b < ctx->buckets.size(); b++) {
            int s = ctx->list_off[b], e = ctx->list_off[b + 1];
            for (int s0 = s; s0 < e; s0 += kChunk) {
                cb.push_back(s0);
                ce.push_back(std::min(e, s0 + kChunk));
                cbk.push_back((int)b);
                per_read++;
            }
        }
        tile_read.reserve((size_t)R * per_read);
        for (int r = 0; r < R; r++) {
            for (int k = 0; k < per_read; k++) {
                tile_read.push_back(r);
                tile_begin.push_back(cb[k]);
                tile_end.push_back(ce[k]);
                tile_bucket.push_back(cbk[k]);
            }
            read_tile_off[r + 1] = (int)tile_read.size();
        }
    }
    const int ntiles = (int)tile_read.size();
    // Order tiles by bucket so that each launch gets a contiguous range.
    std::vector<int> order(ntiles);
    for (int i = 0; i < ntiles; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return tile_bucket[x] < tile_bucket[y]; });
    // Tile arrays in launch order; partial outputs are written at the tile's
    // original index (read-major) so that read_tile_off indexes them.
    std::vector<int> t_read(ntiles), t_begin(ntiles), t_end(ntiles), t_out(ntiles);
    for (int i = 0; i < ntiles; i++) {
        t_read[i] = tile_read[order[i]];
        t_begin[i] = tile_begin[order[i]];
        t_end[i] = tile_end[order[i]];
        t_out[i] = order[i];
    }
    WP_CUDA(ctx->d_tiles.ensure(sizeof(int) * 4 * std::max(ntiles, 1)), "alloc tiles");
    int* d_t = ctx->d_tiles.as<int>();
    WP_CUDA(cudaMemcpyAsync(d_t, t_read.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, ctx->stream), "tiles");
    WP_CUDA(cudaMemcpyAsync(d_t + ntiles, t_begin.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, ctx->stream), "tiles");
    WP_CUDA(cudaMemcpyAsync(d_t + 2 * ntiles, t_end.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, ctx->stream), "tiles");
    WP_CUDA(cudaMemcpyAsync(d_t + 3 * ntiles, t_out.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, ctx->stream), "tiles");
    if (h_cand) {
        WP_CUDA(ctx->d_cand_list.ensure(sizeof(int) * std::max<size_t>(cand_list.size(), 1)), "alloc cand");
        WP_CUDA(ctx->d_cand_key.ensure(sizeof(int) * std::max<size_t>(cand_key.size(), 1)), "alloc cand");
        WP_CUDA(cudaMemcpyAsync(ctx->d_cand_list.p, cand_list.data(), sizeof(int) * cand_list.size(),
                                cudaMemcpyHostToDevice, ctx->stream), "cand");
        WP_CUDA(cudaMemcpyAsync(ctx->d_cand_key.p, cand_key.data(), sizeof(int) * cand_key.size(),
                                cudaMemcpyHostToDevice, ctx->stream), "cand");
        a.list = ctx->d_cand_list.as<int>();
        a.key = ctx->d_cand_key.as<int>();
    } else {
        a.list = ctx->d_list.as<int>();
        a.key = ctx->d_list.as<int>();  // key = peptide index
    }
    WP_CUDA(ctx->d_part_key.ensure(sizeof(int) * std::max(ntiles, 1)), "alloc partials");
    WP_CUDA(ctx->d_part_pep.ensure(sizeof(int) * std::max(ntiles, 1)), "alloc partials");
    WP_CUDA(ctx->d_part_mant.ensure(sizeof(float) * std::max(ntiles, 1)), "alloc partials");
    WP_CUDA(ctx->d_part_expo.ensure(sizeof(int) * std::max(ntiles, 1)), "alloc partials");
    WP_CUDA(ctx->d_part_total.ensure(sizeof(double) * std::max(ntiles, 1)), "alloc partials");
    a.part_key = ctx->d_part_key.as<int>();
    a.part_pep = ctx->d_part_pep.as<int>();
    a.part_mant = ctx->d_part_mant.as<float>();
    a.part_expo = ctx->d_part_expo.as<int>();
    a.part_total = ctx->d_part_total.as<double>();
    // One launch per bucket.
    int i0 = 0;
    while (i0 < ntiles) {
        int b = tile_bucket[order[i0]];
        int i1 = i0;
        while (i1 < ntiles && tile_bucket[order[i1]] == b) i1++;
        int S_cap = ctx->buckets[b].S_cap;
        int warps = warps_for(ctx, S_cap);
        if (warps < 1)
            return fail(ctx, WP_ERR_UNSUPPORTED, "peptide state (" + std::to_string(S_cap) + " x " +
                                                         std::to_string(T) + ") exceeds shared memory");
        size_t smem = wp_forward_smem_bytes(T, S_cap, C, hb, warps);
        TileArgs la = a;
        la.S_cap = S_cap;
        la.tile_read = d_t + i0;
        la.tile_begin = d_t + ntiles + i0;
        la.tile_end = d_t + 2 * ntiles + i0;
        la.tile_out = d_t + 3 * ntiles + i0;
        {
            TimedLaunch tl(ctx, 0);
            WP_CUDA(wp_launch_forward(hb, i1 - i0, warps * 32, smem, ctx->stream, la), "forward launch");
        }
        ctx->launches++;
        i0 = i1;
    }
    if (classify) {
        WP_CUDA(ctx->d_read_tile_off.ensure(sizeof(int) * (R + 1)), "alloc offsets");
        WP_CUDA(cudaMemcpyAsync(ctx->d_read_tile_off.p, read_tile_off.data(), sizeof(int) * (R + 1),
                                cudaMemcpyHostToDevice, ctx->stream), "offsets");
        int threads = 128;
        int blocks = (R + threads - 1) / threads;
        if (blocks > 0) {
            TimedLaunch tl(ctx, 2);
            wp_combine_kernel<<<blocks, threads, 0, ctx->stream>>>(
                    R, ctx->d_read_tile_off.as<int>(), a.part_key, a.part_pep, a.part_mant,
                    a.part_expo, a.part_total, ctx->d_ids.as<int>(), d_out_id, d_out_score,
                    d_out_total, d_out_log);
            ctx->launches++;
            WP_CUDA(cudaGetLastError(), "combine launch");
        }
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
    if (err) return fail(ctx, WP_ERR_CUDA, "internal: peptide state exceeded its bucket");
    return WP_OK;
}

}  // namespace

extern "C" {

wp_status wp_ctx_create(wp_ctx** out, int device) {
    if (!out) return WP_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || device < 0 || device >= n)
        return WP_ERR_CUDA;
    wp_ctx* ctx = new (std::nothrow) wp_ctx();
    if (!ctx) return WP_ERR_OOM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
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
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* wp_last_error(const wp_ctx* ctx) {
    return ctx ? ctx->err.c_str() : "null context";
}

long long wp_launch_count(const wp_ctx* ctx) {
    return ctx ? ctx->launches : 0;
}

void* wp_ctx_stream(const wp_ctx* ctx) {
    return ctx ? (void*)ctx->stream : nullptr;
}

wp_status wp_timing_enable(wp_ctx* ctx, int enable) {
    if (!ctx) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    collect_timing(ctx);
    for (int k = 0; k < 4; k++) {
        ctx->t_ms[k] = 0.0;
        ctx->t_n[k] = 0;
    }
    ctx->timing = enable != 0;
    return WP_OK;
}

wp_status wp_timing_read(wp_ctx* ctx, int kind, double* total_ms, long long* launches) {
    if (!ctx || kind < 0 || kind > 3) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    collect_timing(ctx);
    if (total_ms) *total_ms = ctx->t_ms[kind];
    if (launches) *launches = ctx->t_n[kind];
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

wp_status wp_model_upload(wp_ctx* ctx, const wp_seq_model* m, int T) {
    if (!ctx || !m) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    const int C = m->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS) return fail(ctx, WP_ERR_UNSUPPORTED, "num_channels out of range 1..4");
    if (T < 1 || T > WP_MAX_TIMESTEPS) return fail(ctx, WP_ERR_UNSUPPORTED, "num_timesteps out of range 1..64");
    if (!m->p_bleach || !m->p_dud || !m->bg_sig || !m->mu || !m->sig)
        return fail(ctx, WP_ERR_INVALID, "null per-channel array");
    DevModel& h = ctx->hm;
    memset(&h, 0, sizeof(h));
    h.C = C;
    h.T = T;
    h.pf = (float)m->p_edman_failure;
    h.p_ib = (float)m->p_initial_block;
    h.p_cb = (float)m->p_cyclic_block;
    h.has_block = (m->p_initial_block != 0.0 || m->p_cyclic_block != 0.0) ? 1 : 0;
    for (int t = 0; t < T; t++)  // DecayingRateModel (decaying-rate-model.cc:47-50)
        h.p_det[t] = (float)(m->p_detach + m->p_initial_detach * std::exp(-(double)t * m->p_initial_detach_decay));
    h.interacting = 0;
    for (int c = 0; c < C; c++) {
        binomial_table(m->p_dud[c], WP_MAX_DYES_PER_CHANNEL, h.dud[c]);
        binomial_table(m->p_bleach[c], WP_MAX_DYES_PER_CHANNEL, h.bleach[c]);
        h.bg_sig[c] = m->bg_sig[c];
        h.sig[c] = m->sig[c];
        h.mu[c] = m->mu[c];
        for (int o = 0; o < C; o++) {
            h.inter[c][o] = m->interactions ? m->interactions[c * C + o] : 1.0;
            h.flat[c][o] = m->flat_interactions ? m->flat_interactions[c * C + o] : 1.0;
            if (h.inter[c][o] != 1.0 || h.flat[c][o] != 1.0) h.interacting = 1;
        }
    }
    WP_CUDA(cudaMemcpyAsync(ctx->d_model.p, &h, sizeof(DevModel), cudaMemcpyHostToDevice, ctx->stream),
            "copy model");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync model");
    ctx->have_model = true;
    ctx->plan_C = ctx->plan_T = -1;
    return WP_OK;
}

wp_status wp_peptides_upload(wp_ctx* ctx, const int16_t* dye_seqs, const int32_t* offsets,
                             const int32_t* ids, const int32_t* counts, int P) {
    if (!ctx || P < 0 || (P > 0 && (!offsets || !ids || !counts))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (offsets[0] != 0) return fail(ctx, WP_ERR_INVALID, "offsets[0] must be 0");
    for (int i = 0; i < P; i++)
        if (offsets[i + 1] < offsets[i]) return fail(ctx, WP_ERR_INVALID, "offsets not ascending");
    int n = offsets[P];
    if (n > 0 && !dye_seqs) return WP_ERR_INVALID;
    ctx->seqs.assign(dye_seqs, dye_seqs + n);
    ctx->offsets.assign(offsets, offsets + P + 1);
    ctx->ids.assign(ids, ids + P);
    ctx->counts.assign(counts, counts + P);
    ctx->P = P;
    ctx->have_peps = true;
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
    const int T = ctx->hm.T, C = ctx->hm.C;
    size_t rbytes = sizeof(double) * (size_t)R * T * C;
    WP_CUDA(ctx->d_rads.ensure(rbytes), "alloc reads");
    WP_CUDA(cudaMemcpyAsync(ctx->d_rads.p, rads, rbytes, cudaMemcpyHostToDevice, ctx->stream), "copy reads");
    WP_CUDA(ctx->d_out_id.ensure(sizeof(int32_t) * R), "alloc out");
    WP_CUDA(ctx->d_out_score.ensure(sizeof(double) * R), "alloc out");
    WP_CUDA(ctx->d_out_total.ensure(sizeof(double) * R), "alloc out");
    WP_CUDA(ctx->d_out_log.ensure(sizeof(double) * R), "alloc out");
    st = run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, cand, cand_off, nullptr,
                   ctx->d_out_id.as<int32_t>(), ctx->d_out_score.as<double>(),
                   ctx->d_out_total.as<double>(), ctx->d_out_log.as<double>());
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_id, ctx->d_out_id.p, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    WP_CUDA(cudaMemcpyAsync(out_score, ctx->d_out_score.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    WP_CUDA(cudaMemcpyAsync(out_total, ctx->d_out_total.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    if (out_log_score)
        WP_CUDA(cudaMemcpyAsync(out_log_score, ctx->d_out_log.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy out");
    return finish(ctx);
}

wp_status wp_hmm_classify_device(wp_ctx* ctx, const double* d_rads, int R, double dist_cutoff,
                                 int32_t* d_out_id, double* d_out_score, double* d_out_total,
                                 int async) {
    if (!ctx || R < 0 || (R > 0 && (!d_rads || !d_out_id || !d_out_score || !d_out_total))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (R == 0) return WP_OK;
    WP_CUDA(ctx->d_out_log.ensure(sizeof(double) * R), "alloc out");
    st = run_batch(ctx, d_rads, R, dist_cutoff, nullptr, nullptr, nullptr, d_out_id, d_out_score,
                   d_out_total, ctx->d_out_log.as<double>());
    if (st != WP_OK) return st;
    if (async) return WP_OK;
    return finish(ctx);
}

wp_status wp_hmm_loglik_all(wp_ctx* ctx, const double* rads, int R, double dist_cutoff, double* out_logp) {
    if (!ctx || R < 0 || (R > 0 && (!rads || !out_logp))) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    if (R == 0 || ctx->P == 0) return WP_OK;
    const int T = ctx->hm.T, C = ctx->hm.C;
    size_t rbytes = sizeof(double) * (size_t)R * T * C;
    WP_CUDA(ctx->d_rads.ensure(rbytes), "alloc reads");
    WP_CUDA(cudaMemcpyAsync(ctx->d_rads.p, rads, rbytes, cudaMemcpyHostToDevice, ctx->stream), "copy reads");
    size_t lbytes = sizeof(double) * (size_t)R * ctx->P;
    WP_CUDA(ctx->d_logp.ensure(lbytes), "alloc logp");
    st = run_batch(ctx, ctx->d_rads.as<double>(), R, dist_cutoff, nullptr, nullptr,
                   ctx->d_logp.as<double>(), nullptr, nullptr, nullptr, nullptr);
    if (st != WP_OK) return st;
    WP_CUDA(cudaMemcpyAsync(out_logp, ctx->d_logp.p, lbytes, cudaMemcpyDeviceToHost, ctx->stream), "copy logp");
    return finish(ctx);
}

wp_status wp_hmm_count_flops(wp_ctx* ctx, const double* rads, int R, double dist_cutoff, double* out_flops) {
    if (!ctx || R < 0 || !out_flops || (R > 0 && !rads)) return WP_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    wp_status st = check_ready(ctx);
    if (st != WP_OK) return st;
    *out_flops = 0.0;
    if (R == 0 || ctx->P == 0) return WP_OK;
    st = plan_peptides(ctx);
    if (st != WP_OK) return st;
    const int T = ctx->hm.T, C = ctx->hm.C;
    const int W = ctx->dmax + 1;
    const int entries = wp_read_table_entries(T, C, W, ctx->hm.interacting);
    size_t rbytes = sizeof(double) * (size_t)R * T * C;
    WP_CUDA(ctx->d_rads.ensure(rbytes), "alloc reads");
    WP_CUDA(cudaMemcpyAsync(ctx->d_rads.p, rads, rbytes, cudaMemcpyHostToDevice, ctx->stream), "copy reads");
    WP_CUDA(ctx->d_lo.ensure((size_t)R * T * C), "alloc boxes");
    WP_CUDA(ctx->d_hi.ensure((size_t)R * T * C), "alloc boxes");
    WP_CUDA(ctx->d_table.ensure(sizeof(EmitEntry) * (size_t)R * entries), "alloc emission table");
    long n = (long)R * T;
    wp_prep_reads_kernel<<<(int)((n + 127) / 128), 128, 0, ctx->stream>>>(
            ctx->d_model.as<DevModel>(), ctx->d_rads.as<double>(), R, (unsigned)ctx->dmax, dist_cutoff,
            ctx->d_lo.as<uint8_t>(), ctx->d_hi.as<uint8_t>(), ctx->d_table.as<EmitEntry>(), entries);
    ctx->launches++;
    WP_CUDA(ctx->d_flops.ensure(sizeof(double) * R), "alloc flops");
    WP_CUDA(cudaMemsetAsync(ctx->d_flops.p, 0, sizeof(double) * R, ctx->stream), "clear flops");
    long np = (long)R * ctx->P;
    TimedLaunch tl(ctx, 3);
    wp_count_flops_kernel<<<(int)((np + 127) / 128), 128, 0, ctx->stream>>>(
            ctx->d_model.as<DevModel>(), ctx->d_peps.as<PeptideRec>(), ctx->P, ctx->d_lo.as<uint8_t>(),
            ctx->d_hi.as<uint8_t>(), R, ctx->d_flops.as<double>());
    ctx->launches++;
    WP_CUDA(cudaGetLastError(), "flops launch");
    std::vector<double> per(R);
    WP_CUDA(cudaMemcpyAsync(per.data(), ctx->d_flops.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream), "copy flops");
    WP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    double s = 0.0;
    for (double v : per) s += v;
    *out_flops = s;
    return WP_OK;
}

}  // extern "C"
