// Fused DDA line raster -> per-pixel cluster bitset (s2c_dda_cluster_bitset).
//
// Same bits as the reference's dda_compute_fragments followed by
// cluster_mask_from_fragments (dda.cu:9-256, rasterize.cu:474-520), without a fragment
// list and without global atomics in the common case.  Launches, all on one stream:
//
//  init     zero the per-call counters.
//  bin      one CTA per chunk of 2048 primitives.  Each warp walks 32 segments in
//           lockstep, one fragment per step, with the reference's exact FP32 arithmetic
//           (bounds and depth tests included; the depth test is skipped where both end
//           points are provably inside the clip volume).  Accepted fragments are encoded
//           as runs: one 8-byte entry holds the cluster, the first pixel inside a screen
//           tile and one bit per further step along the minor axis, so a run needs no
//           floating point to replay.  Entries are grouped by tile in shared memory
//           (hash of tile ids, a shared counter per tile whose atomicAdd gives each entry
//           its place), written contiguously per tile, and one (tile, start, count, rank)
//           record per touched tile goes to a record pool.
//  scan     exclusive offsets of the per-tile record counts.
//  scatter  records sorted by tile (each carries its rank in the tile from the bin pass);
//           tiles with many entries listed first.
//  raster   persistent CTAs (3 per SM) take tiles from a queue (heavy ones first):
//           replay the tile's entries into a shared-memory copy of its bitset with
//           atomicOr (a run never leaves its tile, so it walks one shared index), write
//           the whole tile (zeros included) once with coalesced 16-byte streaming stores.
//  fixup    chunks whose entries did not fit (chunk buffer, hash table, entry or record
//           pool) are rasterised with global atomicOr on top of the finished bitset.
#include <algorithm>
#include <climits>

#include "lines.cuh"
#include "scan.cuh"

namespace s2c {

constexpr int kBinThreads = 256;
constexpr int kBinPPT = 8;
constexpr int kChunk = kBinThreads * kBinPPT;  // primitives per bin CTA
constexpr int kHT = 1024;                      // tile hash slots per chunk
constexpr int kStage = 8;                      // staged entries per bin thread
constexpr int kSpill = 1024;                   // shared spill entries per chunk
constexpr int kRasterThreads = 512;
constexpr int kMaxRun = 28;                    // fragments per entry (27 step bits)
constexpr int kHeavy = 8192;                   // entries that make a tile "heavy"

enum { H_ENT = 0, H_REC = 1, H_OVER = 2, H_WORK = 4, H_HEAVY = 5, H_WORDS = 16 };

struct Geo {
    int B, H, W, S;
    int twl, thl;  // log2 tile width / height
    int tiles_x, tiles_y;
    int num_tiles;
};

struct Ws {
    long long* hdr;
    int32_t* nrec;      // records per tile
    int32_t* nent;      // entries per tile
    int32_t* roff;      // exclusive record offsets (inclusive scan, then shifted on use)
    int32_t* heavy;     // heavy tile list
    int32_t* over;      // overflowed chunk ids
    int4* recs;         // (tile, start, count, rank among the tile's records)
    int2* sorted;       // (start, count) grouped by tile
    uint2* entries;
    void* scan_ws;      // scan scratch
    int64_t scan_total_off;
    int64_t entry_cap, rec_cap, chunk_cap;
};

static Geo make_geo(int B, int H, int W, int S) {
    Geo g;
    g.B = B; g.H = H; g.W = W; g.S = S;
    // <= 64 KiB of bitset per tile, >= 64 px, and enough tiles to spread over the GPU
    const int64_t cap_px = std::max<int64_t>(64, std::min<int64_t>(4096, 16384 / std::max(S, 1)));
    const int64_t want = 4LL * num_sms();
    int lg = 6;
    while ((1LL << (lg + 1)) <= cap_px && ((int64_t)B * H * W) >> (lg + 1) >= want) ++lg;
    g.twl = (lg + 1) / 2;
    g.thl = lg / 2;
    g.tiles_x = (W + (1 << g.twl) - 1) >> g.twl;
    g.tiles_y = (H + (1 << g.thl) - 1) >> g.thl;
    g.num_tiles = (int)((int64_t)B * g.tiles_x * g.tiles_y);
    return g;
}

// Workspace layout; with base == nullptr only the sizes are computed.
static size_t layout(void* base, size_t bytes, int64_t P, const Geo& g, Ws& w) {
    Carver c(base, bytes);
    const int64_t T = g.num_tiles;
    w.hdr = c.take<long long>(H_WORDS);
    w.nrec = c.take<int32_t>(T);
    w.nent = c.take<int32_t>(T);
    w.roff = c.take<int32_t>(T);
    w.heavy = c.take<int32_t>(T);
    w.chunk_cap = std::max<int64_t>((P + kChunk - 1) / kChunk, 1);
    w.over = c.take<int32_t>(w.chunk_cap);
    w.rec_cap = std::max<int64_t>(P / 4, 1 << 16);
    w.recs = c.take<int4>(w.rec_cap);
    w.sorted = c.take<int2>(w.rec_cap);
    w.scan_ws = c.take<char>(scan_workspace_bytes(T) + 256);
    w.scan_total_off = (int64_t)scan_workspace_bytes(T);
    const size_t fixed = align_up(c.off, 256);
    w.entries = (uint2*)(c.base + fixed);
    w.entry_cap = bytes > fixed ? std::min<int64_t>((int64_t)((bytes - fixed) / sizeof(uint2)), 0x7fffffffLL) : 0;
    return fixed;
}

__global__ void fused_init(long long* hdr, int32_t* nrec, int32_t* nent, int T) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < H_WORDS) hdr[i] = 0;
    for (int t = i; t < T; t += gridDim.x * blockDim.x) {
        nrec[t] = 0;
        nent[t] = 0;
    }
}

__device__ __forceinline__ int ht_slot(int* keys, int key) {
    unsigned h = ((unsigned)key * 2654435761u) >> 22;  // 10 bits
    for (int probe = 0; probe < kHT; ++probe) {
        const int k = ((volatile int*)keys)[h];
        if (k == key) return (int)h;
        if (k == -1) {
            const int old = atomicCAS(keys + h, -1, key);
            if (old == -1 || old == key) return (int)h;
        }
        h = (h + 1) & (kHT - 1);
    }
    return -1;
}

// cluster of edge e, -1 where the id or the cluster is out of range (the primitive is
// skipped); the reference carries the prim id as float(e + 1)
__device__ __forceinline__ int cluster_of(const int32_t* __restrict__ p2c, int e, int E, int S) {
    const int pr = prim_roundtrip(e);
    if (pr < 0 || pr >= E) return -1;
    const int c = __ldg(p2c + pr);
    return c >= 0 && c < 32 * S ? c : -1;
}

// A primitive with its cluster entry; craw = p2c[prim_roundtrip(e)], or INT_MIN where that
// id is outside [0, E).
struct Lane {
    bool valid;
    int craw;
    Prim q;
};

// Two-stage prefetch (the checks of load_prim, split): the edge (vertex pair) two primitives
// ahead, then its positions and cluster entry one primitive ahead, so that no load waits on
// another inside an iteration.
struct PreEdge {
    bool valid;
    int b, e;
    int2 ev;
};

__device__ __forceinline__ PreEdge fetch_edge(int64_t p, int64_t P, const Lines& L) {
    PreEdge r;
    r.valid = false;
    r.b = 0;
    r.e = 0;
    r.ev = make_int2(0, 0);
    if (p < P) {
        const int64_t eid = L.edge_ids ? (int64_t)__ldg(L.edge_ids + p) : p;
        if (eid >= 0 && eid < L.BE) {
            r.b = L.BE == L.E ? 0 : (int)L.divE.div((uint32_t)eid);
            r.e = (int)eid - r.b * L.E;
            r.ev = __ldg(L.edges2 + r.e);
            r.valid = true;
        }
    }
    return r;
}

__device__ __forceinline__ Lane fetch_pos(const PreEdge& r, const Lines& L, const int32_t* __restrict__ p2c) {
    Lane l;
    l.valid = r.valid && (unsigned)r.ev.x < (unsigned)L.V && (unsigned)r.ev.y < (unsigned)L.V;
    l.q.b = r.b;
    l.q.e = r.e;
    l.craw = INT_MIN;
    if (l.valid) {
        const int64_t vb = (int64_t)r.b * L.V;
        l.q.p0 = __ldg(L.pos4 + vb + r.ev.x);
        l.q.p1 = __ldg(L.pos4 + vb + r.ev.y);
        const int pr = prim_roundtrip(r.e);
        if (pr >= 0 && pr < L.E) l.craw = __ldg(p2c + pr);
    }
    return l;
}

// floor(x) for |x| < 2^22 without a conversion instruction: x + 1.5 * 2^23 rounded down is
// an integer in [2^23, 2^24), whose bits less those of 1.5 * 2^23 are floor(x)
__device__ __forceinline__ int floor_small(float x) { return __float_as_int(__fadd_rd(x, 12582912.0f)) - 0x4B400000; }

// cluster_of on a prefetched entry
__device__ __forceinline__ int cluster_checked(int craw, int S) { return craw >= 0 && craw < 32 * S ? craw : -1; }

__global__ void __launch_bounds__(kBinThreads) dda_bin_kernel(int64_t P, Lines L, Geo g, const int32_t* __restrict__ p2c,
                                                              Ws w) {
    extern __shared__ int smem[];
    int* ht_key = smem;
    int* ht_cnt = ht_key + kHT;
    int* ht_base = ht_cnt + kHT;
    // lane-private staging, entry i of thread t at [i * kBinThreads + t] (conflict-free)
    uint2* st_pay = (uint2*)(ht_base + kHT);                              // kStage * kBinThreads
    uint32_t* st_key = (uint32_t*)(st_pay + kStage * kBinThreads);        // slot | tick << 10
    uint2* sp_pay = (uint2*)(st_key + kStage * kBinThreads);              // shared spill area
    uint32_t* sp_key = (uint32_t*)(sp_pay + kSpill);
    __shared__ int s_spill, s_over, s_nslots, s_reserved, s_total;
    __shared__ long long s_base, s_rbase;
    __shared__ int wb[32];

    for (int i = threadIdx.x; i < kHT; i += blockDim.x) {
        ht_key[i] = -1;
        ht_cnt[i] = 0;
    }
    if (threadIdx.x == 0) {
        s_spill = 0;
        s_over = 0;
        s_reserved = 0;
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int64_t chunk0 = (int64_t)blockIdx.x * kChunk;
    const int TW = 1 << g.twl, TH = 1 << g.thl;
    int n_st = 0;                  // staged entries of this thread
    int last_tile = -1, last_slot = -1;
    auto emit = [&](int tile, uint2 pay) {
        int slot = last_slot;
        if (tile != last_tile) {
            slot = ht_slot(ht_key, tile);
            if (slot < 0) { s_over = 1; return; }
            last_tile = tile;
            last_slot = slot;
        }
        const int tick = atomicAdd(ht_cnt + slot, 1);
        const uint32_t key = (uint32_t)slot | ((uint32_t)tick << 10);
        if (n_st < kStage) {
            st_pay[n_st * kBinThreads + threadIdx.x] = pay;
            st_key[n_st * kBinThreads + threadIdx.x] = key;
            ++n_st;
        } else {
            const int i = atomicAdd(&s_spill, 1);
            if (i < kSpill) {
                sp_pay[i] = pay;
                sp_key[i] = key;
            } else {
                s_over = 1;
            }
        }
    };

    Lane cur = fetch_pos(fetch_edge(chunk0 + threadIdx.x, P, L), L, p2c);
    PreEdge pre = fetch_edge(chunk0 + kBinThreads + threadIdx.x, P, L);
    for (int j = 0; j < kBinPPT; ++j) {
        Lane nxt;  // positions of the next primitive (its edge came one iteration ago)
        nxt.valid = false;
        nxt.craw = INT_MIN;
        PreEdge pre2;  // the edge of the primitive after that
        pre2.valid = false;
        if (j + 2 < kBinPPT) pre2 = fetch_edge(chunk0 + (int64_t)(j + 2) * kBinThreads + threadIdx.x, P, L);
        if (j + 1 < kBinPPT) nxt = fetch_pos(pre, L, p2c);
        if (cur.valid) {
            const Span s = dda_span(cur.q.p0, cur.q.p1, g.H, g.W);
            const int c = s.count > 0 ? cluster_checked(cur.craw, g.S) : -1;
            if (c >= 0) {
                const bool zfast = depth_always_passes(cur.q.p0, cur.q.p1);
                const int axis = s.axis != 0.f;
                const uint32_t xbase = (uint32_t)c | ((uint32_t)axis << 28);
                const int tbase = cur.q.b * g.tiles_y;
                // major / minor view of the sweep
                const float smaj = axis ? s.sy : s.sx, smin = axis ? s.sx : s.sy;
                const int nmaj = axis ? g.H : g.W, nmin = axis ? g.W : g.H;
                const int lgmaj = axis ? g.thl : g.twl, lgmin = axis ? g.twl : g.thl;
                const int last = s.count - 1;
                auto sample = [&](int k, int& im, int& in) {
                    const float d = fminf(fmaxf(__fadd_rn((float)k, 0.5f), s.off0), s.off1);
                    im = __float2int_rd(__fadd_rn(smaj, d));
                    in = __float2int_rd(__fadd_rn(smin, __fmul_rn(d, s.slope)));
                };
                int m0, n0, ml, nl;
                sample(0, m0, n0);
                sample(last, ml, nl);
                // Simple sweep: every fragment passes the depth test, both end fragments are
                // inside the image (coordinates are monotonic in k, so all are), and the
                // major pixel is start + k (exact for interior samples d = k + 0.5; checked
                // at both ends).  Then only the minor coordinate needs evaluating, and the
                // interior samples need no clamping (off0 < 1.5 <= k + 0.5 < off1).
                const int dir = s.slope >= 0.f ? 1 : -1;
                bool simple = zfast && isfinite(s.slope) && last <= 32 && m0 == f2i(smaj) && ml == m0 + last &&
                              m0 >= 0 && ml < nmaj && min(n0, nl) >= 0 && max(n0, nl) < nmin && nmin <= (1 << 21);
                // Phase 1: one bit per step k-1 -> k: does the minor pixel move?  Interior
                // samples are d = k + 0.5 exactly; the last fragment was sampled above.  The
                // interior minor coordinates lie between the end ones, inside [0, nmin) with
                // nmin <= 2^21, so floor_small gives __float2int_rd's result.
                uint32_t bits = 0;
                if (simple) {
                    int prev = n0;
                    bool bad = false;
                    float kf = 1.5f;
                    for (int k = 1; k < last; ++k, kf += 1.0f) {
                        const int in = floor_small(__fadd_rn(smin, __fmul_rn(kf, s.slope)));
                        const int dm = in - prev;
                        bits |= (uint32_t)(dm != 0) << (k - 1);
                        bad |= (dm != 0) & (dm != dir);
                        prev = in;
                    }
                    if (last > 0) {
                        const int dm = nl - prev;
                        bits |= (uint32_t)(dm != 0) << (last - 1);
                        bad |= (dm != 0) & (dm != dir);
                    }
                    simple = !bad;
                }
                if (simple) {
                    // Phase 2: cut at screen-tile borders and every kMaxRun fragments.
                    const uint32_t dbit = (uint32_t)(dir < 0) << 29;
                    const int TM = 1 << lgmaj, TN = 1 << lgmin;
                    // end of the piece that starts at fragment k0 (tile border, run cap or the end)
                    auto piece_end = [&](int k0, int mk) {
                        const int jk = m0 + k0;
                        int k1 = min(last + 1, min(k0 + kMaxRun, k0 + TM - (jk & (TM - 1))));
                        const int dist = dir > 0 ? TN - (mk & (TN - 1)) : (mk & (TN - 1)) + 1;
                        uint32_t ahead = k0 >= 32 ? 0u : bits >> k0;  // bit j: step to fragment k0 + j + 1
                        if (__popc(ahead) >= dist) {
                            for (int i = 1; i < dist; ++i) ahead &= ahead - 1u;
                            k1 = min(k1, k0 + __ffs(ahead));          // first fragment in the next tile
                        }
                        return k1;
                    };
                    auto emit_piece = [&](int k0, int k1, int mk) {
                        const int jk = m0 + k0, n = k1 - k0;
                        const uint32_t steps = (n >= 2) ? ((bits >> k0) & ((1u << (n - 1)) - 1u)) : 0u;
                        const int h = axis ? jk : mk, wv = axis ? mk : jk;
                        const int tile = (tbase + (h >> g.thl)) * g.tiles_x + (wv >> g.twl);
                        const int lp = (h & (TH - 1)) * TW + (wv & (TW - 1));
                        emit(tile, make_uint2(xbase | ((uint32_t)lp << 16) | dbit, (uint32_t)(n - 1) | (steps << 5)));
                    };
                    // The first piece: the whole sweep when both end fragments share a tile
                    // (coordinates are monotonic, so every fragment does) and it fits one entry.
                    const bool one = ((m0 ^ ml) >> lgmaj) == 0 && ((n0 ^ nl) >> lgmin) == 0 && last < kMaxRun;
                    int k1 = one ? last + 1 : piece_end(0, n0);
                    emit_piece(0, k1, n0);
                    int k0 = k1;
                    while (k0 <= last) {
                        const uint32_t below = k0 >= 32 ? bits : (bits & ((1u << k0) - 1u));
                        const int mk = n0 + dir * __popc(below);  // minor pixel of fragment k0
                        k1 = piece_end(k0, mk);
                        emit_piece(k0, k1, mk);
                        k0 = k1;
                    }
                } else {
                    // general sweep: every fragment tested as in the reference
                    int r_n = 0, r_tile = -1, r_lp = 0, r_dir = 0, r_lh = 0, r_lw = 0;
                    unsigned r_steps = 0;
                    for (int k = 0; k < s.count; ++k) {
                        float x, y;
                        dda_sample(s, k, x, y);
                        const int h = f2i(floorf(y)), wv = f2i(floorf(x));
                        bool acc = h >= 0 && h < g.H && wv >= 0 && wv < g.W;
                        if (acc && !zfast) {
                            const float t1 = dda_t1(cur.q.p0, cur.q.p1, x, y, s.axis, g.H, g.W);
                            acc = z_ok(dda_z(cur.q.p0, cur.q.p1, t1));
                        }
                        int tile = -1, lh = 0, lw = 0, dmin = 0;
                        bool extend = false;
                        if (acc) {
                            tile = (tbase + (h >> g.thl)) * g.tiles_x + (wv >> g.twl);
                            lh = h & (TH - 1);
                            lw = wv & (TW - 1);
                            if (r_n > 0 && tile == r_tile && r_n < kMaxRun) {
                                const int dmaj = axis ? lh - r_lh : lw - r_lw;
                                dmin = axis ? lw - r_lw : lh - r_lh;
                                extend = dmaj == 1 &&
                                         (dmin == 0 || ((dmin == 1 || dmin == -1) && (r_dir == 0 || dmin == r_dir)));
                            }
                        }
                        if (extend) {
                            if (dmin) {
                                r_steps |= 1u << (r_n - 1);
                                r_dir = dmin;
                            }
                            ++r_n;
                            r_lh = lh;
                            r_lw = lw;
                            continue;
                        }
                        if (r_n > 0)
                            emit(r_tile, make_uint2(xbase | ((uint32_t)r_lp << 16) | ((uint32_t)(r_dir < 0) << 29),
                                                    (uint32_t)(r_n - 1) | (r_steps << 5)));
                        r_n = 0;
                        if (acc) {
                            r_n = 1;
                            r_tile = tile;
                            r_lp = lh * TW + lw;
                            r_dir = 0;
                            r_steps = 0;
                            r_lh = lh;
                            r_lw = lw;
                        }
                    }
                    if (r_n > 0)
                        emit(r_tile, make_uint2(xbase | ((uint32_t)r_lp << 16) | ((uint32_t)(r_dir < 0) << 29),
                                                (uint32_t)(r_n - 1) | (r_steps << 5)));
                }
            }
        }
        cur = nxt;
        pre = pre2;
    }
    __syncthreads();
    // exclusive scans over the slots: entry offsets and record ranks (4 slots per thread)
    int v[4], used[4], sv = 0, su = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        v[j] = ht_cnt[threadIdx.x * 4 + j];
        used[j] = v[j] > 0;
        sv += v[j];
        su += used[j];
    }
    const int packed = min(sv, 0xffff) | (su << 16);
    int inc = packed;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    const int warp = threadIdx.x >> 5;
    if (lane == 31) wb[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int x = lane < (kBinThreads >> 5) ? wb[lane] : 0;
        int xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += t;
        }
        if (lane < (kBinThreads >> 5)) wb[lane] = xi - x;
        if (lane == (kBinThreads >> 5) - 1) {
            s_nslots = xi >> 16;
            s_total = xi & 0xffff;
        }
    }
    __syncthreads();
    int run = wb[warp] + inc - packed;
    int ebase[4], rrank[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        ebase[j] = run & 0xffff;
        rrank[j] = run >> 16;
        ht_base[threadIdx.x * 4 + j] = ebase[j];
        run += v[j] | (used[j] << 16);
    }
    if (threadIdx.x == 0 && !s_over) {
        const long long b = atomicAdd((unsigned long long*)(w.hdr + H_ENT), (unsigned long long)s_total);
        const long long r = atomicAdd((unsigned long long*)(w.hdr + H_REC), (unsigned long long)s_nslots);
        s_base = b;
        s_rbase = r;
        s_reserved = 1;
        if (b + s_total > w.entry_cap || r + s_nslots > w.rec_cap) s_over = 1;
    }
    __syncthreads();
    if (s_over) {
        // record slots reserved by this chunk stay in the pool: mark them empty
        if (s_reserved)
            for (long long r = s_rbase + threadIdx.x; r < min(s_rbase + s_nslots, (long long)w.rec_cap); r += blockDim.x)
                w.recs[r] = make_int4(-1, 0, 0, 0);
        if (threadIdx.x == 0) {
            const long long o = atomicAdd((unsigned long long*)(w.hdr + H_OVER), 1ull);
            if (o < w.chunk_cap) w.over[o] = (int32_t)blockIdx.x;
        }
        return;
    }
    const long long base = s_base;
    for (int i = 0; i < n_st; ++i) {
        const uint32_t key = st_key[i * kBinThreads + threadIdx.x];
        w.entries[base + ht_base[key & 1023] + (key >> 10)] = st_pay[i * kBinThreads + threadIdx.x];
    }
    const int nsp = min(s_spill, kSpill);
    for (int i = threadIdx.x; i < nsp; i += blockDim.x) {
        const uint32_t key = sp_key[i];
        w.entries[base + ht_base[key & 1023] + (key >> 10)] = sp_pay[i];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (!used[j]) continue;
        const int tile = ht_key[threadIdx.x * 4 + j];
        // the count before this record is its rank among the tile's records
        const int rank = atomicAdd(w.nrec + tile, 1);
        w.recs[s_rbase + rrank[j]] = make_int4(tile, (int)(base + ebase[j]), v[j], rank);
        atomicAdd(w.nent + tile, v[j]);
    }
}

// records -> grouped by tile (roff holds the inclusive scan of nrec); heavy tiles listed
__global__ void __launch_bounds__(256) scatter_records(Ws w, int T) {
    const long long nr = min(w.hdr[H_REC], (long long)w.rec_cap);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t r = i0; r < nr; r += stride) {
        const int4 rc = w.recs[r];
        if (rc.x < 0 || rc.x >= T) continue;  // slot of a chunk that overflowed
        const int pos = w.roff[rc.x] - w.nrec[rc.x] + rc.w;
        w.sorted[pos] = make_int2(rc.y, rc.z);
    }
    for (int64_t t = i0; t < T; t += stride)
        if (w.nent[t] >= kHeavy) w.heavy[atomicAdd((unsigned long long*)(w.hdr + H_HEAVY), 1ull)] = (int)t;
}

__global__ void __launch_bounds__(kRasterThreads, 3) dda_tile_raster_kernel(Geo g, Ws w, int32_t* __restrict__ bitset) {
    extern __shared__ uint32_t sm_bits[];
    const int TW = 1 << g.twl, TH = 1 << g.thl, TPX = TW * TH, S = g.S;
    const int rowstride = TPX + 1;
    __shared__ int s_item, s_rec;
    const bool vec4 = (S & 3) == 0;
    const int n_heavy = (int)w.hdr[H_HEAVY];
    const int items = n_heavy + g.num_tiles;
    const int lane = threadIdx.x & 31;
    // the tile bitset starts cleared; each tile's write-out clears the words it reads
    {
        uint4* z4 = reinterpret_cast<uint4*>(sm_bits);
        const int n4 = (S * rowstride) >> 2;
        for (int i = threadIdx.x; i < n4; i += blockDim.x) z4[i] = make_uint4(0, 0, 0, 0);
        for (int i = (n4 << 2) + threadIdx.x; i < S * rowstride; i += blockDim.x) sm_bits[i] = 0u;
    }
    // The 16-byte stores of a full tile: when a tile row's TW * G items divide the CTA's
    // threads, thread t always takes pixel px and slot group sg (from t mod TW * G) and rows
    // r0, r0 + dR, ... (dR = threads / (TW * G)), so its shared and global offsets are a base
    // plus a fixed stride per store, computed once.  Other shapes and border tiles take the
    // general loop.
    const int G = S >> 2;
    const bool fast_out = vec4 && TW * G <= kRasterThreads && kRasterThreads % (TW * G) == 0 &&
                          (int64_t)TH * g.W * S < (1LL << 31);
    int f_r0 = 0, f_soff = 0, f_goff = 0, f_dr = 1;
    if (fast_out) {
        const int rem = threadIdx.x % (TW * G);
        const int px = rem / G, sg = rem - px * G;
        f_r0 = threadIdx.x / (TW * G);
        f_dr = kRasterThreads / (TW * G);
        f_soff = (4 * sg) * rowstride + f_r0 * TW + px;
        f_goff = (f_r0 * g.W + px) * S + 4 * sg;
    }
    const int f_sstep = f_dr * TW;
    const int64_t f_gstep = (int64_t)f_dr * g.W * S;

    for (;;) {
        if (threadIdx.x == 0) {
            s_item = (int)atomicAdd((unsigned long long*)(w.hdr + H_WORK), 1ull);
            s_rec = 0;
        }
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= items) break;
        int tile;
        if (item < n_heavy) {
            tile = w.heavy[item];
        } else {
            tile = item - n_heavy;
            if (w.nent[tile] >= kHeavy) continue;  // done among the heavy ones
        }
        const int tx = tile % g.tiles_x;
        const int ty = (tile / g.tiles_x) % g.tiles_y;
        const int b = tile / (g.tiles_x * g.tiles_y);
        const int h0 = ty * TH, w0 = tx * TW;
        const int rows = min(TH, g.H - h0), cols = min(TW, g.W - w0);
        const int nrec = w.nrec[tile];
        const int rbeg = w.roff[tile] - nrec;
        const int64_t row0 = ((int64_t)b * g.H + h0) * g.W + w0;
        const bool full = fast_out && rows == TH && cols == TW;
        if (nrec == 0) {
            // empty tile: zeros, 16 bytes per store where possible
            if (full) {
                int32_t* t = bitset + row0 * S + f_goff;
                for (int r = f_r0; r < TH; r += f_dr, t += f_gstep)
                    __stcs(reinterpret_cast<int4*>(t), make_int4(0, 0, 0, 0));
            } else if (vec4) {
                const int per_row = cols * (S >> 2);
                int r = threadIdx.x / per_row, c = threadIdx.x - r * per_row;
                const int dr = kRasterThreads / per_row, dc = kRasterThreads - dr * per_row;
                for (; r < rows;) {
                    __stcs(reinterpret_cast<int4*>(bitset + (row0 + (int64_t)r * g.W) * S) + c, make_int4(0, 0, 0, 0));
                    r += dr;
                    c += dc;
                    if (c >= per_row) { c -= per_row; ++r; }
                }
            } else {
                const int per_row = cols * S;
                int r = threadIdx.x / per_row, c = threadIdx.x - r * per_row;
                const int dr = kRasterThreads / per_row, dc = kRasterThreads - dr * per_row;
                for (; r < rows;) {
                    __stcs(bitset + (row0 + (int64_t)r * g.W) * S + c, 0);
                    r += dr;
                    c += dc;
                    if (c >= per_row) { c -= per_row; ++r; }
                }
            }
            continue;
        }
        // Warps pull records from a shared counter.  Each lane replays one entry of 32: the
        // first four fragments unrolled, longer runs lane by lane.  The next 32 entries (of
        // this record, or the first of the warp's next record) are loaded before the current
        // ones are replayed.
        int r = 0;
        if (lane == 0) r = atomicAdd(&s_rec, 1);
        r = __shfl_sync(0xffffffffu, r, 0);
        int2 rc = r < nrec ? w.sorted[rbeg + r] : make_int2(0, 0);
        uint2 e = (r < nrec && lane < rc.y) ? __ldcs(w.entries + rc.x + lane) : make_uint2(0, 0);
        while (r < nrec) {
            int rn = 0;
            if (lane == 0) rn = atomicAdd(&s_rec, 1);
            rn = __shfl_sync(0xffffffffu, rn, 0);
            const int2 rcn = rn < nrec ? w.sorted[rbeg + rn] : make_int2(0, 0);
            for (int base = 0; base < rc.y; base += 32) {
                uint2 en = make_uint2(0, 0);
                if (base + 32 < rc.y) {
                    if (base + 32 + lane < rc.y) en = __ldcs(w.entries + rc.x + base + 32 + lane);
                } else if (rn < nrec && lane < rcn.y) {
                    en = __ldcs(w.entries + rcn.x + lane);
                }
                int n = 0;
                if (base + lane < rc.y) {
                    n = (int)(e.y & 31) + 1;
                    if ((int)(e.x & 0xffff) >= 32 * S) n = 0;
                }
                const int c = e.x & 0xffff;
                uint32_t* col = sm_bits + (size_t)(c >> 5) * rowstride;
                const uint32_t bit = 1u << (c & 31);
                const int axis = (e.x >> 28) & 1, dir = (e.x >> 29) & 1 ? -1 : 1;
                const unsigned steps = e.y >> 5;
                // Every fragment of an entry lies in the tile (the bin pass cuts runs at tile
                // borders), so a run walks one shared index: one pixel (x-major) or one tile row
                // (y-major) per step, plus the minor move where the step bit is set.
                const int inc_maj = axis ? TW : 1, inc_min = axis ? dir : dir * TW;
                int pix = (e.x >> 16) & 0xfff;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (i < n && (unsigned)pix < (unsigned)TPX) atomicOr(col + pix, bit);
                    pix += inc_maj + (((steps >> i) & 1) ? inc_min : 0);
                }
                for (int i = 4; i < n; ++i) {  // the longer runs, lane by lane
                    if ((unsigned)pix < (unsigned)TPX) atomicOr(col + pix, bit);
                    pix += inc_maj + (((steps >> i) & 1) ? inc_min : 0);
                }
                e = en;
            }
            if (rc.y <= 0) e = (rn < nrec && lane < rcn.y) ? __ldcs(w.entries + rcn.x + lane) : make_uint2(0, 0);
            r = rn;
            rc = rcn;
        }
        __syncthreads();
        if (full) {
            int32_t* t = bitset + row0 * S + f_goff;
            uint32_t* src = sm_bits + f_soff;
            for (int r = f_r0; r < TH; r += f_dr, t += f_gstep, src += f_sstep) {
                const int4 v = make_int4((int)src[0], (int)src[rowstride], (int)src[2 * rowstride], (int)src[3 * rowstride]);
                src[0] = 0u;
                src[rowstride] = 0u;
                src[2 * rowstride] = 0u;
                src[3 * rowstride] = 0u;
                __stcs(reinterpret_cast<int4*>(t), v);
            }
        } else if (vec4) {
            // thread -> (row, pixel, 16-byte slot group), advanced without divisions
            const int per_row = cols * G;
            int r = threadIdx.x / per_row, rem = threadIdx.x - r * per_row;
            const int dr = kRasterThreads / per_row, drem = kRasterThreads - dr * per_row;
            int px = rem / G, sg = rem - px * G;
            const int dpx = drem / G, dsg = drem - dpx * G;
            for (; r < rows;) {
                uint32_t* src = sm_bits + (size_t)(4 * sg) * rowstride + r * TW + px;
                const int4 v = make_int4((int)src[0], (int)src[rowstride], (int)src[2 * rowstride], (int)src[3 * rowstride]);
                src[0] = 0u;
                src[rowstride] = 0u;
                src[2 * rowstride] = 0u;
                src[3 * rowstride] = 0u;
                __stcs(reinterpret_cast<int4*>(bitset + (row0 + (int64_t)r * g.W + px) * S + 4 * sg), v);
                r += dr;
                px += dpx;
                sg += dsg;
                if (sg >= G) { sg -= G; ++px; }
                if (px >= cols) { px -= cols; ++r; }
            }
        } else {
            const int per_row = cols * S;
            for (int i = threadIdx.x; i < rows * per_row; i += blockDim.x) {
                const int r = i / per_row, rem = i - r * per_row;
                const int px = rem / S, sl = rem - px * S;
                uint32_t* src = sm_bits + (size_t)sl * rowstride + r * TW + px;
                const int v = (int)*src;
                *src = 0u;
                __stcs(bitset + (row0 + (int64_t)r * g.W) * S + rem, v);
            }
        }
        __syncthreads();
    }
}

// chunks that did not fit: global atomicOr on the finished bitset
__global__ void __launch_bounds__(256) dda_fixup_kernel(int64_t P, Lines L, Geo g, const int32_t* __restrict__ p2c,
                                                        Ws w, int32_t* __restrict__ bitset) {
    const int64_t noc = min((long long)w.chunk_cap, w.hdr[H_OVER]);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < noc * kChunk; i += stride) {
        const int64_t p = (int64_t)w.over[i / kChunk] * kChunk + (i % kChunk);
        Prim q;
        if (p >= P || !load_prim(p, L, q)) continue;
        const Span s = dda_span(q.p0, q.p1, g.H, g.W);
        const int c = cluster_of(p2c, q.e, L.E, g.S);
        if (c < 0) continue;
        for (int k = 0; k < s.count; ++k) {
            float x, y;
            dda_sample(s, k, x, y);
            const int h = f2i(floorf(y)), wv = f2i(floorf(x));
            if (h < 0 || h >= g.H || wv < 0 || wv >= g.W) continue;
            const float t1 = dda_t1(q.p0, q.p1, x, y, s.axis, g.H, g.W);
            if (!z_ok(dda_z(q.p0, q.p1, t1))) continue;
            atomicOr(bitset + (((int64_t)q.b * g.H + h) * g.W + wv) * g.S + (c >> 5), (int32_t)(1u << (c & 31)));
        }
    }
}

static size_t bin_smem() { return (size_t)3 * kHT * 4 + (size_t)(kStage * kBinThreads + kSpill) * (8 + 4); }
static size_t raster_smem(const Geo& g) { return (size_t)g.S * (((size_t)1 << (g.twl + g.thl)) + 1) * 4; }

}  // namespace s2c

using namespace s2c;

extern "C" size_t s2c_dda_cluster_bitset_workspace_size(int64_t P, int B, int H, int W, int S) {
    if (B <= 0 || H <= 0 || W <= 0 || S <= 0 || P < 0) return 0;
    const Geo g = make_geo(B, H, W, S);
    Ws w;
    const size_t fixed = layout(nullptr, (size_t)-1, P, g, w);
    const int64_t entries = 2 * P + (1 << 16);  // ~1.2 runs per hair segment; 2x headroom
    return fixed + (size_t)entries * sizeof(uint2);
}

namespace s2c {
// host-side argument checks of both bitset entries (no CUDA call)
static s2c_status check_bitset_call(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V, const float* pos,
                                    int E, const int32_t* edges, const int32_t* p2c, int S, const int32_t* bitset,
                                    const char* who) {
    if (s2c_status s = check_lines(P, edge_ids, H, W, B, V, pos, E, edges, who)) return s;
    S2C_REQUIRE(S > 0 && S <= 2048, "%s: slot count must be in [1, 2048] (K <= 65536)", who);
    S2C_REQUIRE(bitset && ((uintptr_t)bitset & 15) == 0, "%s: bitset must be 16-byte aligned", who);
    S2C_REQUIRE(P == 0 || p2c, "%s: null prim2cluster", who);
    const Geo g = make_geo(B, H, W, S);
    S2C_REQUIRE((int64_t)B * g.tiles_x * g.tiles_y < (1LL << 31), "%s: too many tiles", who);
    return S2C_OK;
}
}  // namespace s2c

extern "C" s2c_status s2c_dda_cluster_bitset(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V,
                                             const float* pos, int E, const int32_t* edges, const int32_t* p2c,
                                             int S, int32_t* bitset, void* ws, size_t ws_bytes, s2c_stream stream) {
    if (s2c_status s = check_bitset_call(P, edge_ids, H, W, B, V, pos, E, edges, p2c, S, bitset, "dda_cluster_bitset"))
        return s;
    const Geo g = make_geo(B, H, W, S);
    Ws w;
    const size_t fixed = layout(ws, ws_bytes, P, g, w);
    if (!ws || ws_bytes < fixed + 4096 * sizeof(uint2)) {
        set_error("dda_cluster_bitset: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    const size_t rs = raster_smem(g);
    S2C_REQUIRE(rs <= 200 * 1024, "dda_cluster_bitset: tile too large for shared memory");
    cudaStream_t st = (cudaStream_t)stream;
    // kernel attributes and the raster's occupancy belong to a device: cached per device
    static std::atomic<size_t> cfg_raster[kMaxDevices];
    static std::atomic<bool> cfg_bin[kMaxDevices];
    static std::atomic<int> occ_cache[kMaxDevices];
    static std::atomic<size_t> occ_rs[kMaxDevices];
    const int slot = current_device_slot();
    if (rs > cfg_raster[slot].load()) {
        cudaFuncSetAttribute(dda_tile_raster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs);
        cfg_raster[slot].store(rs);
    }
    if (!cfg_bin[slot].load()) {
        cudaFuncSetAttribute(dda_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bin_smem());
        cfg_bin[slot].store(true);
    }
    const int T = g.num_tiles;
    fused_init<<<grid_for(std::max(T, (int)H_WORDS), 256, 2048), 256, 0, st>>>(w.hdr, w.nrec, w.nent, T);
    S2C_CHECK_LAUNCH("fused_init");
    const Lines L = make_lines(edge_ids, B, V, pos, E, edges);
    if (P > 0) {
        dda_bin_kernel<<<(unsigned)w.chunk_cap, kBinThreads, bin_smem(), st>>>(P, L, g, p2c, w);
        S2C_CHECK_LAUNCH("dda_bin_kernel");
    }
    if (s2c_status s = inclusive_scan_i32(w.nrec, T, w.roff, w.scan_ws, (int64_t*)((char*)w.scan_ws + w.scan_total_off),
                                          st))
        return s;
    scatter_records<<<2 * num_sms(), 256, 0, st>>>(w, T);
    S2C_CHECK_LAUNCH("scatter_records");
    int occ = occ_cache[slot].load();
    if (occ_rs[slot].load() != rs || occ < 1) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dda_tile_raster_kernel, kRasterThreads, rs);
        if (occ < 1) occ = 1;
        occ_cache[slot].store(occ);
        occ_rs[slot].store(rs);
    }
    const unsigned rgrid = (unsigned)std::min<int64_t>((int64_t)occ * num_sms(), T);
    dda_tile_raster_kernel<<<rgrid, kRasterThreads, rs, st>>>(g, w, bitset);
    S2C_CHECK_LAUNCH("dda_tile_raster_kernel");
    if (P > 0) {
        dda_fixup_kernel<<<2 * num_sms(), 256, 0, st>>>(P, L, g, p2c, w, bitset);
        S2C_CHECK_LAUNCH("dda_fixup_kernel");
    }
    return S2C_OK;
}

extern "C" s2c_status s2c_dda_cluster_bitset_stats(const void* ws, size_t ws_bytes, int64_t* entries,
                                                   int64_t* overflow_prims) {
    S2C_REQUIRE(ws && ws_bytes >= H_WORDS * sizeof(long long), "dda_cluster_bitset_stats: bad workspace");
    long long hdr[H_WORDS];
    cudaError_t e = cudaMemcpy(hdr, ws, sizeof(hdr), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "dda_cluster_bitset_stats");
    if (entries) *entries = hdr[H_ENT];
    if (overflow_prims) *overflow_prims = hdr[H_OVER] * kChunk;
    return S2C_OK;
}

// ---------------------------------------------------------------------------------------
// Fixed-scratch variant: the same fused DDA -> bitset with its scratch in a device array
// owned by the library, for callers that cannot allocate device memory themselves (for
// example a plugin running inside a host application that owns the device memory pool
// and hands it only input and output buffers, or a C caller with no allocator to draw a
// workspace from).
// ---------------------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr size_t kFixedScratchBytes = size_t(32) << 20;  // 32 MiB per GPU, held until exit

// Every GPU that loads libs2c.so holds this array for the life of the process.
__device__ __align__(256) unsigned char g_fixed_scratch[kFixedScratchBytes];

std::mutex g_fixed_mu;
void* g_fixed_ptr[256];  // device address of g_fixed_scratch, per device ordinal

// The host symbol g_fixed_scratch is not a device address; cudaGetSymbolAddress gives the
// device address, once per device, with that device current.
s2c_status fixed_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "dda_cluster_bitset_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= 256) {
        set_error("dda_cluster_bitset_noalloc: device ordinal %d out of range", dev);
        return S2C_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_fixed_mu);
    if (!g_fixed_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_fixed_scratch);
        if (e != cudaSuccess) return cuda_status(e, "dda_cluster_bitset_noalloc: cudaGetSymbolAddress");
        g_fixed_ptr[dev] = p;
    }
    *out = g_fixed_ptr[dev];
    return S2C_OK;
}

}  // namespace

extern "C" s2c_status s2c_dda_cluster_bitset_noalloc(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V,
                                                     const float* pos, int E, const int32_t* edges,
                                                     const int32_t* p2c, int S, int32_t* bitset,
                                                     s2c_stream stream) {
    // every argument check before the first CUDA call, as the workspace entry does
    if (s2c_status s = check_bitset_call(P, edge_ids, H, W, B, V, pos, E, edges, p2c, S, bitset,
                                         "dda_cluster_bitset_noalloc"))
        return s;
    const size_t need = s2c_dda_cluster_bitset_workspace_size(P, B, H, W, S);
    if (need > kFixedScratchBytes) {
        set_error("dda_cluster_bitset_noalloc: this problem needs %zu bytes of scratch, more than the fixed %zu "
                  "(use s2c_dda_cluster_bitset with a caller workspace)",
                  need, kFixedScratchBytes);
        return S2C_ERR_INVALID;
    }
    void* scratch = nullptr;
    if (s2c_status s = fixed_scratch(&scratch)) return s;
    // the counters the kernels need zeroed are cleared by the first launch of every call
    return s2c_dda_cluster_bitset(P, edge_ids, H, W, B, V, pos, E, edges, p2c, S, bitset, scratch,
                                  kFixedScratchBytes, stream);
}
