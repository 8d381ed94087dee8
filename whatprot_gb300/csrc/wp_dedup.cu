// wp_dedup.cu -- dye-track dedup on the device: dedup_dye_tracks
// (simulation/dedup-dye-tracks.cc:35-141), which the reference runs as a
// MapReduce-MPI job keyed on the track's counts.  Here it is a sort:
//
//   pack      each instance's T x C counts into W words of `bits`-bit fields,
//             most significant first (word-major [W][n]), and its source id
//   sort      stable LSD radix sorts of an instance permutation: by source
//             id (or with the id folded into word W-1), then by word W-1,
//             ..., word 0 (CUB onesweep), so that the permutation orders
//             instances by (track, id, instance index)
//   flag      first sorted instance of each distinct track and of each
//             (track, id) run; with drop_zero, the all-zero track (the
//             undetectable instances that generate_dye_tracks drops,
//             generate-dye-tracks.cc:52-64) sorts first and gets none
//   scan      inclusive sums of the flags number the tracks and sources
//   scatter   distinct tracks (unpacked to int16), CSR offsets, source id and
//             the count of the id's first instance (the reduce keeps the
//             count of the first value, dedup-dye-tracks.cc:119-124)
//   hits      run lengths of the (track, id) runs
//
// The result is canonical: tracks in lexicographic order of their counts,
// sources of a track in ascending id (the reference's order is that of its
// hash tables).  Every step is a bandwidth-bound pass over n instances; the
// sorts move (8 + 4) bytes per instance per digit pass.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cub/cub.cuh>

#include "wp_common.cuh"

namespace {

// Packs fields into words in track order (field f of word w at bits
// [64 - bits (f + 1), 64 - bits f)).
struct FieldPacker {
    DedupArgs& a;
    int i, w = 0, f = 0, k;
    uint64_t word = 0;
    __device__ FieldPacker(DedupArgs& a_, int i_) : a(a_), i(i_), k(64 / a_.bits) {}
    __device__ void push(unsigned v) {
        word |= (uint64_t)v << (64 - a.bits * (f + 1));
        if (++f == k) flush();
    }
    __device__ void flush() {
        if (f == 0) return;
        a.words[(size_t)w * a.n + i] = word;
        w++;
        f = 0;
        word = 0;
    }
};

template <class In>
__global__ void dd_pack_kernel(DedupArgs a, const In* tracks) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const In* tr = tracks + (size_t)i * a.TC;
    FieldPacker fp(a, i);
    if (((size_t)a.TC * sizeof(In)) % 16 == 0) {
        // rows start on 16-byte boundaries: 16-byte loads
        const uint4* v = reinterpret_cast<const uint4*>(tr);
        constexpr int per = 16 / sizeof(In);
        for (int q = 0; q < a.TC / per; q++) {
            const uint4 x = v[q];
            const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
            for (int h = 0; h < per; h++) {
                const uint32_t lane = xs[h * sizeof(In) / 4];
                const int sh = (h * (int)sizeof(In) * 8) & 31;
                fp.push((lane >> sh) & (sizeof(In) == 1 ? 0xffu : 0xffffu));
            }
        }
    } else {
        for (int j = 0; j < a.TC; j++) fp.push((unsigned)(uint16_t)tr[j]);
    }
    fp.flush();
    int id;
    if (a.pep) {
        const int p = a.pep[i];
        id = p >= 0 ? a.pep_ids[p] : (int)a.id_min;
        a.inst_id[i] = id;
        a.inst_cnt[i] = p >= 0 ? a.pep_cnts[p] : 0;
    } else {
        id = a.inst_id[i];
    }
    if (a.fold_id)
        a.words[(size_t)(a.W - 1) * a.n + i] |= (uint64_t)(uint32_t)((long long)id - a.id_min) << a.id_shift;
    else  // signed id -> unsigned key of the same order
        reinterpret_cast<uint32_t*>(a.keys0)[i] = (uint32_t)id ^ 0x80000000u;
    a.perm0[i] = i;
}

// Word w of instance e without the folded id bits.
__device__ __forceinline__ uint64_t dd_word(const DedupArgs& a, int w, int e) {
    const uint64_t x = a.words[(size_t)w * a.n + e];
    return w == a.W - 1 ? (x & a.last_mask) : x;
}

__global__ void dd_gather_kernel(const uint64_t* word, const int* perm, uint64_t* keys, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = word[perm[i]];
}

__global__ void dd_flag_kernel(DedupArgs a, const int* perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int e = perm[i];
    int ft = 0, fs = 0;
    bool drop = a.drop_zero;
    for (int w = 0; w < a.W && drop; w++) drop = dd_word(a, w, e) == 0;
    if (!drop) {
        if (i == 0) {
            ft = fs = 1;
        } else {
            const int pe = perm[i - 1];
            for (int w = 0; w < a.W && !ft; w++) ft = dd_word(a, w, e) != dd_word(a, w, pe);
            fs = ft || a.inst_id[e] != a.inst_id[pe];
        }
    }
    a.flag_t[i] = ft;
    a.flag_s[i] = fs;
}

__global__ void dd_scatter_kernel(DedupArgs a, const int* perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if (!a.flag_s[i]) return;
    const int e = perm[i];
    const int s = a.scan_s[i] - 1;
    a.start[s] = i;
    a.out_src_id[s] = a.inst_id[e];
    a.out_src_count[s] = a.inst_cnt[e];
    if (!a.flag_t[i]) return;
    const int u = a.scan_t[i] - 1;
    a.out_src_off[u] = s;
    // unpack the fields in track order, stored 8 at a time (16 bytes) when
    // the rows start on 16-byte boundaries
    const int k = 64 / a.bits;
    const uint64_t mask = (1ull << a.bits) - 1;
    int16_t* out = a.out_counts + (size_t)u * a.TC;
    const bool vec = (a.TC * 2) % 16 == 0;
    int w = 0, f = 0;
    uint64_t word = a.words[e];
    uint32_t pack[4];
    for (int j = 0; j < a.TC; j++) {
        const uint32_t v = (uint32_t)((word >> (64 - a.bits * (f + 1))) & mask);
        if (++f == k && j + 1 < a.TC) {
            f = 0;
            word = a.words[(size_t)(++w) * a.n + e];
        }
        if (vec) {
            const int h = j & 7;
            if (h & 1) pack[h >> 1] |= v << 16;
            else pack[h >> 1] = v;
            if (h == 7) reinterpret_cast<uint4*>(out)[j >> 3] = make_uint4(pack[0], pack[1], pack[2], pack[3]);
        } else {
            out[j] = (int16_t)v;
        }
    }
}

__global__ void dd_hits_kernel(DedupArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int U = a.scan_t[a.n - 1], S = a.scan_s[a.n - 1];
    if (s == 0) {
        a.out_src_off[U] = S;
        a.out_sizes[0] = U;
        a.out_sizes[1] = S;
    }
    if (s < S) a.out_src_hits[s] = (s + 1 < S ? a.start[s + 1] : a.n) - a.start[s];
}

// Smallest and largest count over n x TC int16 values (for the field width).
__global__ void dd_range_kernel(const int16_t* c, size_t total, int* minmax) {
    int lo = INT32_MAX, hi = INT32_MIN;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        lo = min(lo, (int)c[i]);
        hi = max(hi, (int)c[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&minmax[0], lo);
        atomicMax(&minmax[1], hi);
    }
}

inline unsigned blocks_for(long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

size_t wp_dedup_temp_bytes(int n) {
    size_t a = 0, b = 0, c = 0;
    cub::DoubleBuffer<uint64_t> k64(nullptr, nullptr);
    cub::DoubleBuffer<uint32_t> k32(nullptr, nullptr);
    cub::DoubleBuffer<int> v(nullptr, nullptr);
    cub::DeviceRadixSort::SortPairs(nullptr, a, k64, v, n);
    cub::DeviceRadixSort::SortPairs(nullptr, b, k32, v, n);
    cub::DeviceScan::InclusiveSum(nullptr, c, (const int*)nullptr, (int*)nullptr, n);
    return std::max(a, std::max(b, c));
}

cudaError_t wp_launch_dedup_range(const int16_t* c, size_t total, int* minmax, cudaStream_t s) {
    // bytes 0x7f.. / 0x80.. start the minimum above and the maximum below
    // every int16 value
    cudaError_t e = cudaMemsetAsync(minmax, 0x7f, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(minmax + 1, 0x80, sizeof(int), s);
    if (e != cudaSuccess || total == 0) return e;
    const unsigned grid = (unsigned)std::min<size_t>((total + 255) / 256, 152 * 8);
    dd_range_kernel<<<grid, 256, 0, s>>>(c, total, minmax);
    return cudaGetLastError();
}

// The whole pipeline on stream s; a.n >= 1.  Launches 5 + W kernels, W + 1
// radix sorts and 2 scans.
cudaError_t wp_launch_dedup(const DedupArgs& a, cudaStream_t s, int* launches) {
    const int T = 256;
    const unsigned g = blocks_for(a.n, T);
    cudaError_t e;
    if (a.in_u8) dd_pack_kernel<uint8_t><<<g, T, 0, s>>>(a, a.in_u8);
    else dd_pack_kernel<int16_t><<<g, T, 0, s>>>(a, a.in_i16);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int nl = 1;
    size_t tb = a.temp_bytes;
    cub::DoubleBuffer<int> perm(a.perm0, a.perm1);
    if (!a.fold_id) {
        cub::DoubleBuffer<uint32_t> k32(reinterpret_cast<uint32_t*>(a.keys0), reinterpret_cast<uint32_t*>(a.keys1));
        e = cub::DeviceRadixSort::SortPairs(a.temp, tb, k32, perm, a.n, 0, 32, s);
        if (e != cudaSuccess) return e;
    }
    cub::DoubleBuffer<uint64_t> k64(a.keys0, a.keys1);
    const int k = 64 / a.bits;
    for (int w = a.W - 1; w >= 0; w--) {
        dd_gather_kernel<<<g, T, 0, s>>>(a.words + (size_t)w * a.n, perm.Current(), k64.Current(), a.n);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        nl++;
        // the fields of a word sit in its top bits, then the folded id (last
        // word); the bits below are 0
        const int nf = std::min(k, a.TC - w * k);
        const int lo = (a.fold_id && w == a.W - 1) ? a.id_shift : 64 - a.bits * nf;
        tb = a.temp_bytes;
        e = cub::DeviceRadixSort::SortPairs(a.temp, tb, k64, perm, a.n, lo, 64, s);
        if (e != cudaSuccess) return e;
    }
    dd_flag_kernel<<<g, T, 0, s>>>(a, perm.Current());
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    tb = a.temp_bytes;
    if ((e = cub::DeviceScan::InclusiveSum(a.temp, tb, a.flag_t, a.scan_t, a.n, s)) != cudaSuccess) return e;
    tb = a.temp_bytes;
    if ((e = cub::DeviceScan::InclusiveSum(a.temp, tb, a.flag_s, a.scan_s, a.n, s)) != cudaSuccess) return e;
    dd_scatter_kernel<<<g, T, 0, s>>>(a, perm.Current());
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    dd_hits_kernel<<<g, T, 0, s>>>(a);
    nl += 3;
    if (launches) *launches += nl;
    return cudaGetLastError();
}
