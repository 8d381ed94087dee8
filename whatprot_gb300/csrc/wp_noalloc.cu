// wp_noalloc.cu -- classify without allocating memory.
//
// Some callers of this library cannot call cudaMalloc: for example an
// acquisition process that classifies reads as the instrument produces them
// and may not stall the device with an allocation (cudaMalloc can
// synchronise the whole device), or a host that runs the library under a
// memory budget owned by someone else.  wp_hmm_classify_noalloc serves
// them: it runs the same kernels as wp_hmm_classify but keeps every
// intermediate buffer, and the copies of the caller's inputs, in one
// file-scope device array of fixed size, and it creates no context,
// stream or event.  The caller passes host inputs and host outputs.
//
// The array (wp_noalloc_scratch, 64 MiB) is part of the library's device
// image: every GPU that loads the library holds it until the process exits.
// Every call shares it and it keeps the last call's contents; what must
// start at zero (work-list counters, the error flag) is cleared by each
// call.  Calls that overlap on the GPU (from several host threads, or on
// several streams) race on the array; a mutex serialises the calls made
// through this entry point in one process.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>

#include "wp_common.cuh"

#define WP_NOALLOC_SCRATCH_BYTES (64u << 20)
#define WP_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char wp_noalloc_scratch[WP_NOALLOC_SCRATCH_BYTES];

// Kernels shared with the allocating path.
__global__ void wp_prep_reads_kernel(const DevModel*, const double*, int, unsigned, double,
                                     uint8_t*, uint8_t*, EmitEntry*, int);
__global__ void wp_read_summary_kernel(BatchArgs);
__global__ void wp_compact_kernel(BatchArgs);
__global__ void wp_reduce_kernel(BatchArgs, int32_t*, double*, double*, double*, const int*);
cudaError_t wp_launch_engine(int C, bool has_block, int threads, size_t smem, cudaStream_t s,
                             const BatchArgs& a, const int2* in, const int* in_count, int* in_head,
                             int2* out, int* out_count, int slab_half, int scr_floats,
                             int spill_error, int* grid_out);
size_t wp_engine_smem_bytes(int slab_half, int scr_floats, bool has_block, int threads);
cudaError_t wp_launch_dense(bool has_block, int threads, size_t smem, cudaStream_t stream,
                            const BatchArgs& a);
size_t wp_dense_smem_bytes(int T, int S_cap, int C, bool has_block, int warps);

namespace {

std::mutex g_noalloc_mu;
void* g_scratch[WP_NOALLOC_MAX_DEVICES];

// DyeSeqPrecomputations per dye-seq (hmm/precomputations/dye-seq-
// precomputations.cc:20-39), built on the device from the copied dye-seqs.
__global__ void wp_noalloc_peptides_kernel(const int16_t* __restrict__ seqs,
                                           const int32_t* __restrict__ offsets, int P, int C,
                                           PeptideRec* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    PeptideRec rec;
    const int16_t* s = seqs + offsets[i];
    int len = offsets[i + 1] - offsets[i];
    int cnt[WP_MAX_CHANNELS] = {0, 0, 0, 0};
    for (int k = 0; k < len; k++)
        if (s[k] >= 0) cnt[s[k]]++;
    for (int c = 0; c < WP_MAX_CHANNELS; c++) rec.D[c] = (uint8_t)(c < C ? cnt[c] : 0);
    for (int e = 0; e < WP_MAX_TIMESTEPS; e++) {
        int d = e < len ? s[e] : -1;
        rec.dye[e] = (int8_t)d;
        rec.tot[e] = (uint8_t)(d >= 0 ? cnt[d] : 0);  // DyeTrack(e, d)
        if (d >= 0) cnt[d]--;
    }
    wp_pack_peptide(rec);
    out[i] = rec;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" wp_status wp_hmm_classify_noalloc(int device, const wp_seq_model* m, int T,
                                             const int16_t* dye_seqs, const int32_t* offsets,
                                             const int32_t* ids, const int32_t* counts, int P,
                                             const double* rads, int R, double dist_cutoff,
                                             int32_t* out_id, double* out_score, double* out_total) {
    if (!m || R < 0 || P < 1 || !offsets || !ids || !counts) return WP_ERR_INVALID;
    if (R > 0 && (!rads || !out_id || !out_score || !out_total)) return WP_ERR_INVALID;
    if (device < 0 || device >= WP_NOALLOC_MAX_DEVICES) return WP_ERR_INVALID;
    const int C = m->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS || T < 1 || T > WP_MAX_TIMESTEPS) return WP_ERR_UNSUPPORTED;
    if (!m->p_bleach || !m->p_dud || !m->bg_sig || !m->mu || !m->sig) return WP_ERR_INVALID;
    if (offsets[0] != 0 || offsets[P] < 0) return WP_ERR_INVALID;
    if (offsets[P] > 0 && !dye_seqs) return WP_ERR_INVALID;
    // Peptide shape summary on the host, without allocating.
    int dmax = 0, S_max = 1;
    for (int i = 0; i < P; i++) {
        if (offsets[i + 1] < offsets[i]) return WP_ERR_INVALID;
        int cnt[WP_MAX_CHANNELS] = {0, 0, 0, 0};
        for (int k = offsets[i]; k < offsets[i + 1]; k++) {
            int d = dye_seqs[k];
            if (d < -1 || d >= C) return WP_ERR_INVALID;
            if (d >= 0) cnt[d]++;
        }
        int prod = 1;
        for (int c = 0; c < C; c++) {
            if (cnt[c] > WP_MAX_DYES_PER_CHANNEL) return WP_ERR_UNSUPPORTED;
            dmax = cnt[c] > dmax ? cnt[c] : dmax;
            prod *= cnt[c] + 1;
        }
        S_max = prod > S_max ? prod : S_max;
    }
    if (R == 0) return WP_OK;

    // Layout of the scratch array for this call; reject what does not fit.
    DevModel hm;
    const wp_status mst = wp_fill_dev_model(m, T, &hm);
    if (mst != WP_OK) return mst;
    const int W = dmax + 1;
    const int entries = wp_read_table_entries(T, C, W, hm.interacting);
    const long n_slots = (long)R * P;
    const size_t rtc = (size_t)R * T * C;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const size_t o_model = take(sizeof(DevModel));
    const size_t o_peps = take(sizeof(PeptideRec) * P);
    const size_t o_ids = take(sizeof(int) * P);
    const size_t o_counts = take(sizeof(int) * P);
    const size_t o_seqs = take(sizeof(int16_t) * (offsets[P] > 0 ? offsets[P] : 1));
    const size_t o_offsets = take(sizeof(int32_t) * (P + 1));
    const size_t o_rads = take(sizeof(double) * rtc);
    const size_t o_lo = take(rtc), o_hi = take(rtc), o_Ls = take(rtc), o_Up = take(rtc);
    const size_t o_allow = take((size_t)R * T), o_flags = take((size_t)R);
    const size_t o_Lpk = take(sizeof(uint32_t) * (size_t)R * T), o_Upk = take(sizeof(uint32_t) * (size_t)R * T);
    const size_t o_table = take(sizeof(EmitEntry) * (size_t)R * entries);
    const size_t o_mant = take(sizeof(float) * n_slots), o_expo = take(sizeof(int) * n_slots);
    const size_t o_work = take(sizeof(int2) * n_slots), o_ovf1 = take(sizeof(int2) * n_slots),
                 o_ovf2 = take(sizeof(int2) * n_slots);
    const size_t o_cnt = take(sizeof(int) * 8), o_err = take(sizeof(int));
    const size_t o_id = take(sizeof(int32_t) * R), o_sc = take(sizeof(double) * R),
                 o_tot = take(sizeof(double) * R);
    if (off > WP_NOALLOC_SCRATCH_BYTES || n_slots > INT32_MAX) return WP_ERR_UNSUPPORTED;

    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cudaSetDevice(device) != cudaSuccess) return WP_ERR_CUDA;
    // Set-up, once per device: the device address of the scratch array.
    // The first call on a device does this and must come before any stream
    // capture.
    if (!g_scratch[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, wp_noalloc_scratch) != cudaSuccess || !p) return WP_ERR_CUDA;
        g_scratch[device] = p;
    }
    unsigned char* base = static_cast<unsigned char*>(g_scratch[device]);
    cudaStream_t s = 0;  // the legacy default stream: nothing to create
    int dev_attr = 0;
    cudaDeviceGetAttribute(&dev_attr, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    const size_t smem_optin = (size_t)dev_attr;

#define WP_NA(call)                                  \
    do {                                             \
        if ((call) != cudaSuccess) return WP_ERR_CUDA; \
    } while (0)
    WP_NA(cudaMemcpyAsync(base + o_model, &hm, sizeof(DevModel), cudaMemcpyHostToDevice, s));
    WP_NA(cudaMemcpyAsync(base + o_ids, ids, sizeof(int) * P, cudaMemcpyHostToDevice, s));
    WP_NA(cudaMemcpyAsync(base + o_counts, counts, sizeof(int) * P, cudaMemcpyHostToDevice, s));
    if (offsets[P] > 0)
        WP_NA(cudaMemcpyAsync(base + o_seqs, dye_seqs, sizeof(int16_t) * offsets[P], cudaMemcpyHostToDevice, s));
    WP_NA(cudaMemcpyAsync(base + o_offsets, offsets, sizeof(int32_t) * (P + 1), cudaMemcpyHostToDevice, s));
    WP_NA(cudaMemcpyAsync(base + o_rads, rads, sizeof(double) * rtc, cudaMemcpyHostToDevice, s));
    WP_NA(cudaMemsetAsync(base + o_cnt, 0, sizeof(int) * 8, s));
    WP_NA(cudaMemsetAsync(base + o_err, 0, sizeof(int), s));
    wp_noalloc_peptides_kernel<<<(P + 127) / 128, 128, 0, s>>>(
            reinterpret_cast<const int16_t*>(base + o_seqs), reinterpret_cast<const int32_t*>(base + o_offsets),
            P, C, reinterpret_cast<PeptideRec*>(base + o_peps));
    WP_NA(cudaGetLastError());

    BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.model = reinterpret_cast<const DevModel*>(base + o_model);
    a.peps = reinterpret_cast<const PeptideRec*>(base + o_peps);
    a.counts = reinterpret_cast<const int*>(base + o_counts);
    a.R = R;
    a.P = P;
    a.W = W;
    a.entries = entries;
    a.lo = base + o_lo;
    a.hi = base + o_hi;
    a.Lsuf = base + o_Ls;
    a.Upre = base + o_Up;
    a.allow = base + o_allow;
    a.Lpk = reinterpret_cast<uint32_t*>(base + o_Lpk);
    a.Upk = reinterpret_cast<uint32_t*>(base + o_Upk);
    a.flags = base + o_flags;
    a.tab = reinterpret_cast<const EmitEntry*>(base + o_table);
    a.res_mant = reinterpret_cast<float*>(base + o_mant);
    a.res_expo = reinterpret_cast<int*>(base + o_expo);
    a.work = reinterpret_cast<int2*>(base + o_work);
    int* cnt = reinterpret_cast<int*>(base + o_cnt);
    a.work_count = cnt + 0;
    a.work_head = cnt + 1;
    a.ovf = reinterpret_cast<int2*>(base + o_ovf2);
    a.ovf_count = cnt + 4;
    a.ovf_head = cnt + 5;
    a.err = reinterpret_cast<int*>(base + o_err);
    a.dense_S_cap = ((S_max + 31) / 32) * 32;
    const bool hb = hm.has_block != 0;

    wp_prep_reads_kernel<<<(int)(((long)R * T + 127) / 128), 128, 0, s>>>(
            a.model, reinterpret_cast<const double*>(base + o_rads), R, (unsigned)dmax, dist_cutoff,
            base + o_lo, base + o_hi, reinterpret_cast<EmitEntry*>(base + o_table), entries);
    WP_NA(cudaGetLastError());
    wp_read_summary_kernel<<<(R + 127) / 128, 128, 0, s>>>(a);
    WP_NA(cudaGetLastError());
    // Engine passes: the shapes the allocating path uses (two CTAs of 256
    // threads per SM, then one of 128; no per-thread scratch floats, as
    // there), then the dense fallback.
    auto half_for = [&](int threads, int per_sm) {
        size_t budget = smem_optin;
        if (per_sm > 1 && budget > (size_t)(228 * 1024) / per_sm - 1024) budget = (size_t)(228 * 1024) / per_sm - 1024;
        size_t elem = hb ? 8 : 4;
        size_t fixed = wp_engine_smem_bytes(0, 0, hb, threads);
        return budget <= fixed ? 0 : (int)((budget - fixed) / (2 * elem * threads));
    };
    const int half1 = half_for(256, 2), half2 = half_for(128, 1);
    if (half1 < 4 || half2 < 4) return WP_ERR_UNSUPPORTED;
    int dense_warps = 0;
    for (int w = 16; w >= 1; w--)
        if (wp_dense_smem_bytes(T, a.dense_S_cap, C, hb, w) <= smem_optin) {
            dense_warps = w;
            break;
        }
    // the compaction sends each pair to the first pass whose slab holds it
    a.n_tiers = half2 > half1 ? 2 : 1;
    a.tier_half[0] = half1;
    a.tier_list[0] = a.work;
    a.tier_count[0] = cnt + 0;
    a.tier_half[1] = half2;
    a.tier_list[1] = reinterpret_cast<int2*>(base + o_ovf1);
    a.tier_count[1] = cnt + 2;
    a.route_dense = dense_warps > 0 ? 1 : 0;
    wp_compact_kernel<<<R, 256, 0, s>>>(a);
    WP_NA(cudaGetLastError());
    WP_NA(wp_launch_engine(C, hb, 256, wp_engine_smem_bytes(half1, 0, hb, 256), s, a, a.work, cnt + 0,
                           cnt + 1, reinterpret_cast<int2*>(base + o_ovf1), cnt + 2, half1, 0, 0, nullptr));
    WP_NA(wp_launch_engine(C, hb, 128, wp_engine_smem_bytes(half2, 0, hb, 128), s, a,
                           reinterpret_cast<int2*>(base + o_ovf1), cnt + 2, cnt + 3,
                           reinterpret_cast<int2*>(base + o_ovf2), cnt + 4, half2, 0,
                           dense_warps == 0 ? 1 : 0, nullptr));
    if (dense_warps > 0)
        WP_NA(wp_launch_dense(hb, dense_warps * 32, wp_dense_smem_bytes(T, a.dense_S_cap, C, hb, dense_warps), s, a));
    wp_reduce_kernel<<<(R + 3) / 4, 128, 0, s>>>(a, reinterpret_cast<int32_t*>(base + o_id),
                                                 reinterpret_cast<double*>(base + o_sc),
                                                 reinterpret_cast<double*>(base + o_tot), nullptr,
                                                 reinterpret_cast<const int*>(base + o_ids));
    WP_NA(cudaGetLastError());
    WP_NA(cudaMemcpyAsync(out_id, base + o_id, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, s));
    WP_NA(cudaMemcpyAsync(out_score, base + o_sc, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
    WP_NA(cudaMemcpyAsync(out_total, base + o_tot, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
    int err = 0;
    WP_NA(cudaMemcpyAsync(&err, base + o_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    WP_NA(cudaStreamSynchronize(s));
#undef WP_NA
    if (err == 2) return WP_ERR_UNSUPPORTED;
    if (err) return WP_ERR_CUDA;
    return WP_OK;
}
