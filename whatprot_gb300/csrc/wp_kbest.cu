// wp_kbest.cu -- the reference's k-hit set: the kd-tree search with KBest
// (kd-tree/k-best.h:26-42, internal-node.h:39-60, leaf-node.h:31-62)
// replayed on the GPU, one warp per read.
//
// What the reference keeps.  KBest pushes every entry the search offers
// below its current bound kth, then pops the farthest entry if the hits of
// the others still reach k (at most one pop per push), and sets kth to the
// farthest kept distance once the hits reach k.  Until then it keeps
// everything it meets ("fill").  After the fill every pushed entry lies
// below the current farthest one, so the farthest kept entry (the "top")
// only moves down; hence the entries it ends with are exactly those whose
// (squared distance, tree position) is at most the final top's.  The replay
// below runs the same pushes and pops in the same order and returns that
// final top; the entries at or below it are gathered afterwards by the
// brute-force collect pass (wp_nn.cu).
//
// The order of the pushes is the reference's: the tree is walked
// depth-first, nearer child first, the farther child visited when kth is
// above the squared distance to its splitting plane; a leaf's entries are
// met in tree order.  An entry is pushed iff its FP64 squared distance,
// summed as LeafNode::consider sums it (groups of four, then singles), is
// below kth at that moment.  Skipping a whole tile of 32 entries whose
// bounding box lies beyond kth changes nothing (each would be refused).
// Distances are screened in FP32 against kth with a margin that covers the
// FP32 error; the FP64 distance is formed for every entry that passes.
//
// The priority queue.  Since the top only moves down, the replay keeps the
// kept entries in a monotone bucket queue instead of a heap: buckets are
// 1/256-octave ranges of the squared distance (the FP64 exponent and top
// eight mantissa bits, relative to a base), each a chain of 16-entry chunks
// in per-warp global scratch; the bucket of the top is held sorted in shared
// memory ("current bucket").  A push below the current bucket appends to its
// bucket's chain; a pop advances in the current bucket, and when that is
// spent the next non-empty bucket below is loaded and sorted.  The base is
// set so the largest kept entry lies in the highest bucket ("rebase"): at
// the end of the fill, when the walk reaches the catch-all bucket 0, and
// (with 8x narrower buckets) when a bucket holds more entries than the
// current-bucket capacity.  Rebasing copies the live entries into the other
// of two scratch regions, which also reclaims spent chunks when a region
// fills up.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

#define KB_B 2048      // buckets
#define KB_CH 16       // entries per chunk
#define KB_CUR 256     // capacity of the current bucket
#define KB_SHDEF 44    // bucket = FP64 bits >> 44: exponent and 8 mantissa bits
#define KB_SHMIN 20    // narrowest buckets a refinement may reach
#define KB_WARPS 2     // warps per CTA

// Per-warp shared memory (fixed part).
struct KBSmem {
    uint16_t tail[KB_B];   // chain tail chunk of each bucket
    uint8_t fill[KB_B];    // entries in that chunk
    uint32_t ne[KB_B / 32];  // non-empty buckets
    double cd[KB_CUR];     // current bucket, sorted by (d, pos) descending
    int cp[KB_CUR];
    int ch[KB_CUR];
    double q64[64];        // the query
    float q32[64];
    int qpos[64];          // screened entries waiting for their FP64 distances
};

struct KBState {
    long long S;     // hits of the kept entries
    double kth;      // KBest::kth_dist_sq
    int fill_mode;   // hits have not reached k yet
    int cb;          // current bucket (KB_B: none)
    int len, ptr;    // current bucket's entries and the top's index
    long long base;  // bucket origin (FP64 bits >> sh)
    int sh;
    int act;         // active scratch region
    int alloc;       // entries allocated in it
    int fatal;
    double tie_d;    // smallest distance refused for equalling kth
    double top_d;
    int top_pos, top_hits;
};

struct KBCtx {
    const KBArgs* a;
    KBSmem* sm;
    KBItem* reg0;   // region r at reg0 + r * rc (a runtime-indexed array
    int* prev0;     // would live in local memory)
    long rc, pc;
    KBItem* stage;
    int lane;
    __device__ __forceinline__ KBItem* reg(int r) const { return reg0 + r * rc; }
    __device__ __forceinline__ int* prev(int r) const { return prev0 + r * pc; }
};

__device__ __forceinline__ bool kb_gt(double da, int pa, double db, int pb) {
    return da > db || (da == db && pa > pb);
}

__device__ __forceinline__ int kb_bucket(const KBState& st, double d) {
    const long long b = (__double_as_longlong(d) >> st.sh) - st.base;
    return b < 0 ? 0 : (b > KB_B - 1 ? KB_B - 1 : (int)b);
}

__device__ __forceinline__ bool kb_nonempty(const KBSmem* sm, int b) { return (sm->ne[b >> 5] >> (b & 31)) & 1u; }

// Append an entry to bucket b's chain in the active region; false when the
// region is full.
__device__ __forceinline__ bool kb_append(KBCtx& c, KBState& st, int b, double d, int pos, int hits) {
    KBSmem* sm = c.sm;
    const bool ne = kb_nonempty(sm, b);
    int f = ne ? sm->fill[b] : KB_CH;
    int chunk = ne ? sm->tail[b] : 0;
    const int oldtail = chunk;
    bool fresh = false;
    if (f == KB_CH) {
        if (st.alloc + KB_CH > c.a->regcap) return false;
        chunk = st.alloc / KB_CH;
        st.alloc += KB_CH;
        f = 0;
        fresh = true;
    }
    __syncwarp();
    if (c.lane == 0) {
        if (fresh) c.prev(st.act)[chunk] = ne ? oldtail : -1;
        KBItem it;
        it.d = d;
        it.pos = pos;
        it.hits = hits;
        c.reg(st.act)[(long)chunk * KB_CH + f] = it;
        sm->tail[b] = (uint16_t)chunk;
        sm->fill[b] = (uint8_t)(f + 1);
        sm->ne[b >> 5] |= 1u << (b & 31);
    }
    __syncwarp();
    return true;
}

// Every live entry (bucket chains and the rest of the current bucket) into
// the staging buffer; returns their number, or -1 if they do not fit.
__device__ __forceinline__ int kb_gather(KBCtx& c, KBState& st) {
    KBSmem* sm = c.sm;
    const KBItem* reg = c.reg(st.act);
    const int* prev = c.prev(st.act);
    const int cap = c.a->stagecap;
    int n = 0;
    for (int w = 0; w < KB_B / 32; w++) {
        unsigned m = sm->ne[w];
        while (m) {
            const int b = w * 32 + __ffs(m) - 1;
            m &= m - 1;
            int chunk = sm->tail[b], f = sm->fill[b];
            while (chunk >= 0) {
                if (n + f > cap) return -1;
                if (c.lane < f) c.stage[n + c.lane] = reg[(long)chunk * KB_CH + c.lane];
                n += f;
                chunk = prev[chunk];
                f = KB_CH;
            }
        }
    }
    const int rest = st.len - st.ptr;
    if (n + rest > cap) return -1;
    for (int i = c.lane; i < rest; i += 32) {
        KBItem it;
        it.d = sm->cd[st.ptr + i];
        it.pos = sm->cp[st.ptr + i];
        it.hits = sm->ch[st.ptr + i];
        c.stage[n + i] = it;
    }
    n += rest;
    __syncwarp();
    return n;
}

// Redistribute the live entries into the other region with bucket shift
// `sh`, the largest one in the highest bucket.  Leaves no current bucket.
__device__ __forceinline__ void kb_rebase(KBCtx& c, KBState& st, int sh) {
    const int n = kb_gather(c, st);
    if (n < 0) {
        st.fatal = 1;
        return;
    }
    double mx = 0.0;
    for (int i = c.lane; i < n; i += 32) mx = fmax(mx, c.stage[i].d);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    st.act ^= 1;
    st.alloc = 0;
    for (int i = c.lane; i < KB_B / 32; i += 32) c.sm->ne[i] = 0u;
    __syncwarp();
    st.sh = sh;
    st.base = (__double_as_longlong(mx) >> sh) - (KB_B - 1);
    st.cb = KB_B;
    st.len = st.ptr = 0;
    for (int i0 = 0; i0 < n; i0 += 32) {
        KBItem mine;
        mine.d = 0.0;
        mine.pos = 0;
        mine.hits = 0;
        if (i0 + c.lane < n) mine = c.stage[i0 + c.lane];
        const int cnt = min(32, n - i0);
        for (int j = 0; j < cnt; j++) {
            const double d = __shfl_sync(0xffffffffu, mine.d, j);
            const int pos = __shfl_sync(0xffffffffu, mine.pos, j);
            const int hits = __shfl_sync(0xffffffffu, mine.hits, j);
            if (!kb_append(c, st, kb_bucket(st, d), d, pos, hits)) {
                st.fatal = 2;
                return;
            }
        }
    }
}

// Load bucket b as the current bucket, sorted; false (nothing changed) if
// it holds more than KB_CUR entries.
__device__ __forceinline__ bool kb_enter(KBCtx& c, KBState& st, int b) {
    KBSmem* sm = c.sm;
    const KBItem* reg = c.reg(st.act);
    const int* prev = c.prev(st.act);
    int chunk = sm->tail[b], f = sm->fill[b], n = 0;
    while (chunk >= 0) {
        if (n + f > KB_CUR) return false;
        if (c.lane < f) {
            const KBItem it = reg[(long)chunk * KB_CH + c.lane];
            sm->cd[n + c.lane] = it.d;
            sm->cp[n + c.lane] = it.pos;
            sm->ch[n + c.lane] = it.hits;
        }
        n += f;
        chunk = prev[chunk];
        f = KB_CH;
    }
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = n + c.lane; i < n2; i += 32) {
        sm->cd[i] = -1.0;  // below every distance: sorts last
        sm->cp[i] = -1;
        sm->ch[i] = 0;
    }
    __syncwarp();
    // bitonic sort, descending by (d, pos)
    for (int size = 2; size <= n2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = c.lane; i < n2; i += 32) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool desc = (i & size) == 0;
                    const double di = sm->cd[i], dj = sm->cd[j];
                    const int pi = sm->cp[i], pj = sm->cp[j];
                    if (kb_gt(dj, pj, di, pi) == desc) {
                        const int hi = sm->ch[i];
                        sm->cd[i] = dj;
                        sm->cp[i] = pj;
                        sm->ch[i] = sm->ch[j];
                        sm->cd[j] = di;
                        sm->cp[j] = pi;
                        sm->ch[j] = hi;
                    }
                }
            }
            __syncwarp();
        }
    if (c.lane == 0) sm->ne[b >> 5] &= ~(1u << (b & 31));
    __syncwarp();
    st.len = n;
    st.ptr = 0;
    st.cb = b;
    return true;
}

__device__ __forceinline__ void kb_load_top(KBCtx& c, KBState& st) {
    st.top_d = c.sm->cd[st.ptr];
    st.top_pos = c.sm->cp[st.ptr];
    st.top_hits = c.sm->ch[st.ptr];
}

// Make the highest non-empty bucket below the current one current.
__device__ __forceinline__ void kb_descend(KBCtx& c, KBState& st) {
    for (int guard = 0; guard < 64; guard++) {
        const int lim = st.cb;  // buckets < lim
        const int top_w = (lim - 1) >> 5;
        const unsigned top_mask = ((lim - 1) & 31) == 31 ? 0xffffffffu : ((1u << (((lim - 1) & 31) + 1)) - 1u);
        int j = -1;
        for (int w0 = top_w; w0 >= 0 && j < 0; w0 -= 32) {
            const int w = w0 - c.lane;
            unsigned m = 0u;
            if (w >= 0) {
                m = c.sm->ne[w];
                if (w == top_w) m &= top_mask;
            }
            const unsigned any = __ballot_sync(0xffffffffu, m != 0u);
            if (any) {
                const int L = __ffs(any) - 1;
                const unsigned mw = __shfl_sync(0xffffffffu, m, L);
                j = (w0 - L) * 32 + 31 - __clz(mw);
            }
        }
        if (j < 0) {
            st.fatal = 3;
            return;
        }
        if (j == 0 && st.cb != KB_B) {
            // the catch-all bucket: spread what is left again
            kb_rebase(c, st, KB_SHDEF);
            if (st.fatal) return;
            continue;
        }
        if (kb_enter(c, st, j)) return;
        if (st.sh - 3 < KB_SHMIN) {
            st.fatal = 4;
            return;
        }
        kb_rebase(c, st, st.sh - 3);
        if (st.fatal) return;
    }
    st.fatal = 5;
}

__device__ __forceinline__ void kb_pop(KBCtx& c, KBState& st) {
    st.ptr++;
    if (st.ptr == st.len) {
        kb_descend(c, st);
        if (st.fatal) return;
    }
    kb_load_top(c, st);
}

// Insert below the top into the current bucket, keeping it sorted.
__device__ __forceinline__ void kb_cur_insert(KBCtx& c, KBState& st, double d, int pos, int hits) {
    KBSmem* sm = c.sm;
    int at = st.len;
    for (int i0 = st.ptr + 1; i0 < st.len; i0 += 32) {
        const int i = i0 + c.lane;
        const bool below = i < st.len && !kb_gt(sm->cd[i], sm->cp[i], d, pos);
        const unsigned m = __ballot_sync(0xffffffffu, below);
        if (m) {
            at = i0 + __ffs(m) - 1;
            break;
        }
    }
    for (int i1 = st.len - 1; i1 >= at; i1 -= 32) {
        const int i = i1 - c.lane;
        double vd = 0.0;
        int vp = 0, vh = 0;
        const bool mv = i >= at;
        if (mv) {
            vd = sm->cd[i];
            vp = sm->cp[i];
            vh = sm->ch[i];
        }
        __syncwarp();
        if (mv) {
            sm->cd[i + 1] = vd;
            sm->cp[i + 1] = vp;
            sm->ch[i + 1] = vh;
        }
        __syncwarp();
    }
    if (c.lane == 0) {
        sm->cd[at] = d;
        sm->cp[at] = pos;
        sm->ch[at] = hits;
    }
    __syncwarp();
    st.len++;
}

// KBest::insert.
__device__ __forceinline__ void kb_insert(KBCtx& c, KBState& st, double d, int pos, int hits) {
    const long long k = c.a->k;
    st.S += hits;
    if (st.fill_mode) {
        // no base yet: everything goes to bucket 0 until the hits reach k
        if (!kb_append(c, st, 0, d, pos, hits)) {
            st.fatal = 6;
            return;
        }
        if (st.S < k) return;
        st.fill_mode = 0;
        st.cb = KB_B;
        kb_rebase(c, st, KB_SHDEF);
        if (st.fatal) return;
        kb_descend(c, st);
        if (st.fatal) return;
        kb_load_top(c, st);
    } else {
        const int b = kb_bucket(st, d);
        if (b >= st.cb) {
            if (st.len < KB_CUR) {
                kb_cur_insert(c, st, d, pos, hits);
            } else {
                // the current bucket is full: narrower buckets
                if (st.sh - 3 < KB_SHMIN) {
                    st.fatal = 7;
                    return;
                }
                kb_rebase(c, st, st.sh - 3);
                if (st.fatal) return;
                if (!kb_append(c, st, kb_bucket(st, d), d, pos, hits)) {
                    st.fatal = 8;
                    return;
                }
                kb_descend(c, st);
                if (st.fatal) return;
                kb_load_top(c, st);
            }
        } else if (!kb_append(c, st, b, d, pos, hits)) {
            // the region is full: compact into the other one
            kb_rebase(c, st, st.sh);
            if (st.fatal) return;
            if (!kb_append(c, st, kb_bucket(st, d), d, pos, hits)) {
                st.fatal = 9;
                return;
            }
            kb_descend(c, st);
            if (st.fatal) return;
            kb_load_top(c, st);
        }
    }
    if (st.S - st.top_hits >= k) {
        st.S -= st.top_hits;
        kb_pop(c, st);
        if (st.fatal) return;
    }
    st.kth = st.top_d;
}

// A lane's entry row: counts (one byte per coordinate) as 32-bit words.
template <int DP>
__device__ __forceinline__ void kb_row(const uint8_t* __restrict__ cnt, long p, uint32_t (&w)[DP / 4]) {
    const uint4* src = reinterpret_cast<const uint4*>(cnt + p * DP);
#pragma unroll
    for (int i = 0; i < DP / 16; i++) {
        const uint4 v = __ldg(src + i);
        w[4 * i] = v.x;
        w[4 * i + 1] = v.y;
        w[4 * i + 2] = v.z;
        w[4 * i + 3] = v.w;
    }
}

template <int DP>
__device__ __forceinline__ int kb_byte(const uint32_t (&w)[DP / 4], int i) {
    return (int)((w[i >> 2] >> (8 * (i & 3))) & 255u);
}

// FP64 squared distance as LeafNode::consider sums it: groups of four while
// i < D - 3, then single terms; every term from the per-read table
// sq64[i][n] = (q_i - coordinate(i, n))^2.
template <int DP>
__device__ __forceinline__ double kb_d64_tab(const uint32_t (&w)[DP / 4], const double* sq64, int NC, int TC) {
    double acc = 0.0;
#pragma unroll
    for (int i = 0; i < DP; i += 4) {
        if (i + 3 < TC) {
            const double s = __dadd_rn(__dadd_rn(__dadd_rn(sq64[i * NC + kb_byte<DP>(w, i)],
                                                           sq64[(i + 1) * NC + kb_byte<DP>(w, i + 1)]),
                                                 sq64[(i + 2) * NC + kb_byte<DP>(w, i + 2)]),
                                       sq64[(i + 3) * NC + kb_byte<DP>(w, i + 3)]);
            acc = __dadd_rn(acc, s);
        } else {
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (i + u < TC) acc = __dadd_rn(acc, sq64[(i + u) * NC + kb_byte<DP>(w, i + u)]);
        }
    }
    return acc;
}

template <int DP>
__device__ __forceinline__ float kb_d32_tab(const uint32_t (&w)[DP / 4], const float* sq32, int NC, int TC) {
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int i = 0; i < DP; i += 2) {
        if (i < TC) a0 += sq32[i * NC + kb_byte<DP>(w, i)];
        if (i + 1 < TC) a1 += sq32[(i + 1) * NC + kb_byte<DP>(w, i + 1)];
    }
    return a0 + a1;
}

// The same from FP64 coordinates (models with dye interactions).
__device__ __forceinline__ double kb_d64_coords(const double* __restrict__ e, const double* q, int TC) {
    double acc = 0.0;
    int i = 0;
    for (; i + 3 < TC; i += 4) {
        const double x1 = __dsub_rn(q[i], e[i]), x2 = __dsub_rn(q[i + 1], e[i + 1]);
        const double x3 = __dsub_rn(q[i + 2], e[i + 2]), x4 = __dsub_rn(q[i + 3], e[i + 3]);
        const double s = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2)), __dmul_rn(x3, x3)),
                                   __dmul_rn(x4, x4));
        acc = __dadd_rn(acc, s);
    }
    for (; i < TC; i++) {
        const double x = __dsub_rn(q[i], e[i]);
        acc = __dadd_rn(acc, __dmul_rn(x, x));
    }
    return acc;
}

template <int DP, bool INTER>
__global__ void __launch_bounds__(KB_WARPS * 32) wp_kbest_kernel(KBArgs a) {
    extern __shared__ __align__(16) unsigned char kb_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const size_t tab_bytes = INTER ? 0 : ((size_t)a.TC * a.NC * (sizeof(double) + sizeof(float)) + 15) / 16 * 16;
    const size_t stack_bytes = ((size_t)a.stack_cap * (sizeof(int) + sizeof(double)) + 15) / 16 * 16;
    const size_t per_warp = sizeof(KBSmem) + tab_bytes + stack_bytes;
    unsigned char* mine = kb_smem + per_warp * wib;
    KBSmem* sm = reinterpret_cast<KBSmem*>(mine);
    double* sq64 = reinterpret_cast<double*>(mine + sizeof(KBSmem));
    float* sq32 = reinterpret_cast<float*>(sq64 + (INTER ? 0 : a.TC * a.NC));
    double* s_plane = reinterpret_cast<double*>(mine + sizeof(KBSmem) + tab_bytes);
    int* s_node = reinterpret_cast<int*>(s_plane + a.stack_cap);

    const long gw = (long)blockIdx.x * KB_WARPS + wib;
    KBCtx c;
    c.a = &a;
    c.sm = sm;
    c.lane = lane;
    c.rc = a.regcap;
    c.pc = a.regcap / KB_CH;
    c.reg0 = a.reg + gw * 2 * c.rc;
    c.prev0 = a.prev + gw * 2 * c.pc;
    c.stage = a.stage + gw * (long)a.stagecap;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.next, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.nwork) break;
        const int slot = a.work ? a.work[item] : item;
        const int r = a.qperm ? a.qperm[slot] : slot;
        // the query and its per-read distance tables
        for (int i = lane; i < 64; i += 32) {
            const double v = i < a.TC ? a.rads[(long)r * a.TC + i] : 0.0;
            sm->q64[i] = v;
            sm->q32[i] = (float)v;
        }
        __syncwarp();
        if (!INTER) {
            for (int i = lane; i < a.TC * a.NC; i += 32) {
                const int dim = i / a.NC, n = i % a.NC;
                const double x = __dsub_rn(sm->q64[dim], a.ctab[(dim % a.C) * a.NC + n]);
                const double s = __dmul_rn(x, x);
                sq64[i] = s;
                sq32[i] = (float)s;
            }
        }
        __syncwarp();
        KBState st;
        st.S = 0;
        st.kth = DBL_MAX;
        st.fill_mode = 1;
        st.cb = KB_B;
        st.len = st.ptr = 0;
        st.base = 0;
        st.sh = KB_SHDEF;
        st.act = 0;
        st.alloc = 0;
        st.fatal = 0;
        st.tie_d = INFINITY;
        st.top_d = 0.0;
        st.top_pos = -1;
        st.top_hits = 0;
        for (int i = lane; i < KB_B / 32; i += 32) sm->ne[i] = 0u;
        __syncwarp();
        // depth-first walk, nearer child first (InternalNode::search)
        int sp = 0;
        if (lane == 0) {
            s_node[0] = a.N > 0 ? 0 : -1;
            s_plane[0] = -1.0;
        }
        __syncwarp();
        sp = a.N > 0 ? 1 : 0;
        while (sp > 0 && !st.fatal) {
            sp--;
            int node = s_node[sp];
            const double plane = s_plane[sp];
            __syncwarp();
            if (plane >= 0.0 && !(st.kth > plane)) continue;
            KDNode n = a.nodes[node];
            while (!n.leaf) {
                const double qv = sm->q64[n.s];
                int near, far;
                double dist;
                if (qv < n.split) {
                    near = n.left;
                    far = n.right;
                    dist = n.min_right - qv;
                } else {
                    near = n.right;
                    far = n.left;
                    dist = qv - n.max_left;
                }
                if (sp >= a.stack_cap) {
                    st.fatal = 10;
                    break;
                }
                if (lane == 0) {
                    s_node[sp] = far;
                    s_plane[sp] = __dmul_rn(dist, dist);
                }
                __syncwarp();
                sp++;
                node = near;
                n = a.nodes[node];
            }
            if (st.fatal) break;
            // the leaf's entries in tree order
            if (!st.fill_mode) {
                float g2 = 0.f;
                for (int i = lane; i < a.TC; i += 32) {
                    const float lo = a.llo[(long)node * a.DP + i], hi = a.lhi[(long)node * a.DP + i];
                    const float qq = sm->q32[i];
                    const float g = fmaxf(fmaxf(lo - qq, qq - hi), 0.f);
                    g2 = fmaf(g, g, g2);
                }
                for (int o = 16; o > 0; o >>= 1) g2 += __shfl_xor_sync(0xffffffffu, g2, o);
                if ((double)g2 > st.kth * (1.0 + 1e-4) + 1e-3) continue;
            }
            // Tiles of 32 tree positions: each lane screens one entry in FP32
            // (the next tile's counts already loading); entries that may lie
            // below kth join a queue in tree order; 32 queued entries at a
            // time get their FP64 distances (one per lane) and are offered
            // to KBest in order, each against the kth of that moment.
            const long t_lo = n.begin >> 5, t_hi = (long)(n.end - 1) >> 5;
            int qn = 0;
            uint32_t w[DP / 4], wn[DP / 4];
#pragma unroll
            for (int i = 0; i < DP / 4; i++) w[i] = wn[i] = 0u;
            if (!INTER) {
                const long p0 = t_lo * 32 + lane;
                if (p0 >= n.begin && p0 < n.end) kb_row<DP>(a.cnt, p0, w);
            }
            for (long t = t_lo; t <= t_hi && !st.fatal; t++) {
                const long p = t * 32 + lane;
                const bool in = p >= n.begin && p < n.end;
                const long pn = p + 32;
                if (!INTER && t < t_hi && pn >= n.begin && pn < n.end) kb_row<DP>(a.cnt, pn, wn);
                bool cand = false;
                if (in) {
                    if (INTER) {
                        const float* e = a.coords32 + p * a.DP;
                        float acc = 0.f;
                        for (int i = 0; i < a.TC; i++) {
                            const float x = sm->q32[i] - e[i];
                            acc = fmaf(x, x, acc);
                        }
                        cand = st.fill_mode || (double)acc < st.kth * (1.0 + 2e-5) + 1e-3;
                    } else {
                        const float d32 = kb_d32_tab<DP>(w, sq32, a.NC, a.TC);
                        cand = st.fill_mode || (double)d32 < st.kth * (1.0 + 1e-5);
                    }
                }
#pragma unroll
                for (int i = 0; i < DP / 4; i++) w[i] = wn[i];
                const unsigned m = __ballot_sync(0xffffffffu, cand);
                if (cand) sm->qpos[qn + __popc(m & ((1u << lane) - 1u))] = (int)p;
                qn += __popc(m);
                __syncwarp();
                while (qn >= 32 || (t == t_hi && qn > 0)) {
                    const int cnt = min(32, qn);
                    double d64 = 0.0;
                    int h = 0, pos = 0;
                    if (lane < cnt) {
                        pos = sm->qpos[lane];
                        if (INTER) {
                            d64 = kb_d64_coords(a.ecoord + (long)pos * a.TC, sm->q64, a.TC);
                        } else {
                            uint32_t r[DP / 4];
                            kb_row<DP>(a.cnt, pos, r);
                            d64 = kb_d64_tab<DP>(r, sq64, a.NC, a.TC);
                        }
                        h = a.hits[pos];
                    }
                    // the rest of the queue moves to its front
                    int rest = 0;
                    if (lane + cnt < qn) rest = sm->qpos[lane + cnt];
                    __syncwarp();
                    if (lane + cnt < qn) sm->qpos[lane] = rest;
                    __syncwarp();
                    qn -= cnt;
                    for (int j = 0; j < cnt; j++) {
                        const double dj = __shfl_sync(0xffffffffu, d64, j);
                        const int hj = __shfl_sync(0xffffffffu, h, j);
                        const int pj = __shfl_sync(0xffffffffu, pos, j);
                        if (dj < st.kth) {
                            kb_insert(c, st, dj, pj, hj);
                            if (st.fatal) break;
                        } else if (dj == st.kth) {
                            st.tie_d = fmin(st.tie_d, dj);
                        }
                    }
                    if (st.fatal) break;
                }
            }
        }
        if (lane == 0) {
            int flag = 0;
            if (st.fatal) {
                flag = 4 | (st.fatal << 8);
                a.tf_d[slot] = 0.0;
                a.tf_pos[slot] = -1;
            } else if (st.fill_mode) {
                flag = 1;  // the hits never reach k: every entry is kept
                a.tf_d[slot] = INFINITY;
                a.tf_pos[slot] = 0x7fffffff;
            } else {
                if (st.tie_d == st.top_d) flag = 2;
                a.tf_d[slot] = st.top_d;
                a.tf_pos[slot] = st.top_pos;
            }
            a.tf_flag[slot] = flag;
        }
        __syncwarp();
    }
}

int wp_kbest_warps_per_cta() { return KB_WARPS; }
int wp_kbest_chunk() { return KB_CH; }

size_t wp_kbest_smem_bytes(int TC, int NC, int stack_cap, bool inter) {
    const size_t tab = inter ? 0 : ((size_t)TC * NC * (sizeof(double) + sizeof(float)) + 15) / 16 * 16;
    const size_t stk = ((size_t)stack_cap * (sizeof(int) + sizeof(double)) + 15) / 16 * 16;
    return (sizeof(KBSmem) + tab + stk) * KB_WARPS;
}

template <int DP, bool INTER>
static cudaError_t kb_launch(int grid, size_t smem, cudaStream_t s, const KBArgs& a) {
    cudaError_t e = cudaFuncSetAttribute(wp_kbest_kernel<DP, INTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    wp_kbest_kernel<DP, INTER><<<grid, KB_WARPS * 32, smem, s>>>(a);
    return cudaGetLastError();
}

// grid CTAs of KB_WARPS warps; scratch sized for grid * KB_WARPS warps.
cudaError_t wp_launch_kbest(int grid, cudaStream_t s, const KBArgs& a) {
    const size_t smem = wp_kbest_smem_bytes(a.TC, a.NC, a.stack_cap, a.interact != 0);
    if (grid <= 0 || a.nwork == 0) return cudaSuccess;
    if (a.interact) {
        switch (a.DP) {
            case 16: return kb_launch<16, true>(grid, smem, s, a);
            case 32: return kb_launch<32, true>(grid, smem, s, a);
            case 48: return kb_launch<48, true>(grid, smem, s, a);
            case 64: return kb_launch<64, true>(grid, smem, s, a);
        }
    } else {
        switch (a.DP) {
            case 16: return kb_launch<16, false>(grid, smem, s, a);
            case 32: return kb_launch<32, false>(grid, smem, s, a);
            case 48: return kb_launch<48, false>(grid, smem, s, a);
            case 64: return kb_launch<64, false>(grid, smem, s, a);
        }
    }
    return cudaErrorInvalidValue;
}
