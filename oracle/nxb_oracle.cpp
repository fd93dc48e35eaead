// nxb_oracle.cpp - CPU restatement of the NexusBVH build pipeline.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU pipeline is
// compared against and the multithreaded CPU baseline that is timed beside
// it.  Nothing in the product (the CUDA library and its C ABI) links it,
// calls it or falls back to it.
//
// Every stage restates the reference algorithm (paths are inside the
// NexusBVH project; the reference ships no tests, golden vectors or CPU
// path, so parity of this restatement is pinned by fixtures produced by the
// reference's own CUDA build and by GPU probes of the compiler's numerics):
//   scene bounds + leaves   NexusBVH/src/Cuda/Setup.cu:12-39
//   Morton codes            NexusBVH/src/Cuda/Setup.cu:42-59,
//                           NexusBVH/src/Cuda/BuilderUtils.h:104-253
//   stable radix sort       NexusBVH/src/Cuda/Setup.cu:62-112 (CUB 3.0.1
//                           DeviceRadixSort::SortPairs, bits [2,32)/[1,64))
//   H-PLOC                  NexusBVH/src/Cuda/BinaryBuilder.cu:14-273
//   BVH8 collapse           NexusBVH/src/Cuda/WideConverter.cu:104-414
//   cost evaluation         NexusBVH/src/Cuda/Eval.cu:12-80
//
// Floating point: the reference is compiled with --use_fast_math, so every
// float add/sub/mul/min/max flushes subnormal inputs and results to
// sign-preserving zero.  The helpers below apply the same flushing with
// ordinary IEEE arithmetic.  Division is IEEE here (the GPU's fast-math
// divide is not reproduced); Morton codes are therefore compared with a
// documented +-1 tolerance at quantisation boundaries.  Two compiler
// choices that the reference leaves implicit are parameters of this oracle,
// pinned against the GPU by the numerics self-test:
//   * the FMA contraction of AABB::Area (NexusBVH/include/NXB/AABB.h:46-50);
//   * the float -> uint8_t conversion of the BVH8 quantisation
//     (NexusBVH/src/Cuda/WideConverter.cu:195-201).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

struct Box {
    float mn[3];
    float mx[3];
};
struct Node2 {
    Box b;
    uint32_t left;
    uint32_t right;
};
static_assert(sizeof(Node2) == 32, "BVH2 node is 32 bytes");

struct Node8 {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t prim_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(Node8) == 80, "BVH8 node is 80 bytes");

// ------------------------------------------------------------- settings
int g_threads = 0;    // 0 = hardware concurrency
// orc_build's BVH8 stage: 0 = bvh8() (work-slot order), 1 = bvh8_levels()
// (level-parallel; set where the build is timed as the CPU baseline)
int g_level_collapse = 0;
int g_area_form = 2;  // see area()
int g_u8_mode = 0;    // 0: (uint8)(uint32 truncating convert); 1: saturate to [0,255]
int g_min_zero = 0;   // 0: min(+0,-0) = -0 and max = +0 whatever the order

int threads() {
    if (g_threads > 0) return g_threads;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

void parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn, size_t min_chunk = 1 << 14) {
    int t = threads();
    size_t chunks = std::min<size_t>((size_t)t, (n + min_chunk - 1) / min_chunk);
    if (chunks <= 1) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> pool;
    size_t per = (n + chunks - 1) / chunks;
    for (size_t c = 0; c < chunks; ++c) {
        size_t b = c * per, e = std::min(n, b + per);
        if (b >= e) break;
        pool.emplace_back(fn, b, e);
    }
    for (auto& th : pool) th.join();
}

// ------------------------------------------------- fast-math float helpers
inline uint32_t fbits(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
}
inline float bitsf(uint32_t u) {
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}
inline float ftz(float x) {
    uint32_t u = fbits(x);
    if ((u & 0x7F800000u) == 0) u &= 0x80000000u;
    return bitsf(u);
}
inline float fadd(float a, float b) { return ftz(ftz(a) + ftz(b)); }
inline float fsub(float a, float b) { return ftz(ftz(a) - ftz(b)); }
inline float fmul(float a, float b) { return ftz(ftz(a) * ftz(b)); }
inline float ffma(float a, float b, float c) { return ftz(std::fma(ftz(a), ftz(b), ftz(c))); }

// fminf / fmaxf as the GPU evaluates them under -ftz: a NaN operand yields
// the other operand, and -0 orders below +0.
inline float fmin_gpu(float a, float b) {
    a = ftz(a);
    b = ftz(b);
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    if (a < b) return a;
    if (b < a) return b;
    if (g_min_zero == 0) return std::signbit(a) ? a : b;
    return a;
}
inline float fmax_gpu(float a, float b) {
    a = ftz(a);
    b = ftz(b);
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    if (a > b) return a;
    if (b > a) return b;
    if (g_min_zero == 0) return std::signbit(a) ? b : a;
    return a;
}

// AABB::Area (NexusBVH/include/NXB/AABB.h:46-50): dx*dy + dy*dz + dz*dx.
// Form 0: no contraction; 1: fma(dz,dx, fma(dy,dz, dx*dy));
// 2: fma(dz,dx, fma(dx,dy, dy*dz)).
inline float area(const Box& b) {
    float dx = fsub(b.mx[0], b.mn[0]);
    float dy = fsub(b.mx[1], b.mn[1]);
    float dz = fsub(b.mx[2], b.mn[2]);
    switch (g_area_form) {
        case 0: return fadd(fadd(fmul(dx, dy), fmul(dy, dz)), fmul(dz, dx));
        case 1: return ffma(dz, dx, ffma(dy, dz, fmul(dx, dy)));
        default: return ffma(dz, dx, ffma(dx, dy, fmul(dy, dz)));
    }
}

// AABB::Grow(const AABB&) (AABB.h:28-32): this = min/max(this, other).
inline void grow(Box& self, const Box& other) {
    for (int a = 0; a < 3; ++a) {
        self.mn[a] = fmin_gpu(self.mn[a], other.mn[a]);
        self.mx[a] = fmax_gpu(self.mx[a], other.mx[a]);
    }
}

// cvt.rzi.u32.f32: truncate toward zero, NaN and negatives -> 0, saturate.
inline uint32_t f2u_rz(float x) {
    if (std::isnan(x) || x <= 0.0f) return 0;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}
inline uint8_t f2u8(float x) {
    if (g_u8_mode == 1) {
        if (std::isnan(x) || x <= 0.0f) return 0;
        if (x >= 255.0f) return 255;
        return (uint8_t)x;
    }
    return (uint8_t)f2u_rz(x);
}

// ---------------------------------------------------------- stage 1
// ComputeSceneBoundsKernel (Setup.cu:12-39): leaf i = {bounds(prim i),
// INVALID, i}; scene = union of all leaf bounds.  Triangle bounds follow
// AABB(v0,v1,v2) (AABB.h:16-20): min(v0, min(v1, v2)).
void scene_bounds(const float* prims, int prim_type, uint32_t n, Node2* leaves, Box* scene) {
    int nt = threads();
    std::vector<Box> part((size_t)nt + 1);
    std::atomic<int> slot{0};
    parallel_for(n, [&](size_t b, size_t e) {
        Box acc;
        for (int a = 0; a < 3; ++a) {
            acc.mn[a] = 3.402823466e+38f;
            acc.mx[a] = -3.402823466e+38f;
        }
        for (size_t i = b; i < e; ++i) {
            Box bb;
            if (prim_type == 1) {
                const float* t = prims + 9 * i;
                for (int a = 0; a < 3; ++a) {
                    bb.mn[a] = fmin_gpu(t[a], fmin_gpu(t[3 + a], t[6 + a]));
                    bb.mx[a] = fmax_gpu(t[a], fmax_gpu(t[3 + a], t[6 + a]));
                }
            } else {
                const float* t = prims + 6 * i;
                for (int a = 0; a < 3; ++a) {
                    bb.mn[a] = t[a];
                    bb.mx[a] = t[3 + a];
                }
            }
            leaves[i].b = bb;
            leaves[i].left = kInvalid;
            leaves[i].right = (uint32_t)i;
            grow(acc, bb);
        }
        part[slot.fetch_add(1)] = acc;
    });
    Box s;
    for (int a = 0; a < 3; ++a) {
        s.mn[a] = 3.402823466e+38f;
        s.mx[a] = -3.402823466e+38f;
    }
    for (int i = 0; i < slot.load(); ++i) grow(s, part[i]);
    *scene = s;
}

// ---------------------------------------------------------- stage 2
// InterleaveBits32/64 and MortonCode32/64 (BuilderUtils.h:104-226): spread
// the low 10 (21) bits of x three apart; code = x | y<<1 | z<<2.  Written as
// a per-bit loop rather than the magic-mask form.
inline uint32_t spread10(uint32_t x) {
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((x >> b) & 1u) << (3 * b);
    return r;
}
inline uint64_t spread21(uint64_t x) {
    uint64_t r = 0;
    for (int b = 0; b < 21; ++b) r |= ((x >> b) & 1ull) << (3 * b);
    return r;
}

// Quantised normalised centroid (Setup.cu:50-54, BuilderUtils.h:234-253):
// c = (min+max)*0.5; t = (c - smin) / (smax - smin); q = (u32)(t * scale).
inline void quantise(const Box& b, const Box& scene, float scale, uint32_t q[3], float prod[3]) {
    for (int a = 0; a < 3; ++a) {
        float c = fmul(fadd(b.mn[a], b.mx[a]), 0.5f);
        float num = fsub(c, scene.mn[a]);
        float den = fsub(scene.mx[a], scene.mn[a]);
        float t = ftz(ftz(num) / ftz(den));
        float p = fmul(t, scale);
        prod[a] = p;
        q[a] = f2u_rz(p);
    }
}

void morton(const Node2* leaves, uint32_t n, const Box& scene, int key_bits, void* keys, uint32_t* cluster) {
    parallel_for(n, [&](size_t b, size_t e) {
        uint32_t q[3];
        float p[3];
        for (size_t i = b; i < e; ++i) {
            if (key_bits == 30) {
                quantise(leaves[i].b, scene, 1023.0f, q, p);
                ((uint32_t*)keys)[i] = spread10(q[0] & 1023u) | spread10(q[1] & 1023u) << 1 |
                                       spread10(q[2] & 1023u) << 2;
            } else {
                quantise(leaves[i].b, scene, 2097151.0f, q, p);
                ((uint64_t*)keys)[i] = spread21(q[0] & 0x1FFFFFu) | spread21(q[1] & 0x1FFFFFu) << 1 |
                                       spread21(q[2] & 0x1FFFFFu) << 2;
            }
            if (cluster) cluster[i] = (uint32_t)i;
        }
    });
}

// ---------------------------------------------------------- stage 3
// Stable LSD radix sort of (key, value) by key bits [begin, end), 8-bit
// digits, per-thread histograms; identical in result to CUB's SortPairs on
// the same bit range (a stable sort by (key >> begin) & mask).
template <class K>
void radix_sort(const K* kin, const uint32_t* vin, uint32_t n, uint32_t begin, uint32_t end, K* kout,
                uint32_t* vout) {
    std::vector<K> ka(kin, kin + n), kb(n);
    std::vector<uint32_t> va(n), vb(n);
    for (uint32_t i = 0; i < n; ++i) va[i] = vin ? vin[i] : i;
    int nt = std::max(1, std::min(threads(), (int)((n + 65535) / 65536)));
    size_t per = ((size_t)n + nt - 1) / nt;
    std::vector<uint32_t> hist((size_t)nt * 256);
    for (uint32_t bit = begin; bit < end; bit += 8) {
        uint32_t width = std::min(8u, end - bit);
        K mask = (K)((1u << width) - 1);
        std::fill(hist.begin(), hist.end(), 0);
        auto count = [&](int t) {
            size_t b = t * per, e = std::min<size_t>(n, b + per);
            uint32_t* h = &hist[(size_t)t * 256];
            for (size_t i = b; i < e; ++i) h[(ka[i] >> bit) & mask]++;
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(count, t);
        for (auto& th : pool) th.join();
        pool.clear();
        uint32_t run = 0;
        for (int d = 0; d < 256; ++d)
            for (int t = 0; t < nt; ++t) {
                uint32_t c = hist[(size_t)t * 256 + d];
                hist[(size_t)t * 256 + d] = run;
                run += c;
            }
        auto scatter = [&](int t) {
            size_t b = t * per, e = std::min<size_t>(n, b + per);
            uint32_t* h = &hist[(size_t)t * 256];
            for (size_t i = b; i < e; ++i) {
                uint32_t d = (uint32_t)((ka[i] >> bit) & mask);
                uint32_t o = h[d]++;
                kb[o] = ka[i];
                vb[o] = va[i];
            }
        };
        for (int t = 0; t < nt; ++t) pool.emplace_back(scatter, t);
        for (auto& th : pool) th.join();
        ka.swap(kb);
        va.swap(vb);
    }
    std::memcpy(kout, ka.data(), sizeof(K) * n);
    std::memcpy(vout, va.data(), sizeof(uint32_t) * n);
}

// ---------------------------------------------------------- stage 4
// Delta (BinaryBuilder.cu:14-28): xor of neighbouring keys, index-extended.
inline uint64_t delta(const uint32_t* k, uint32_t a, uint32_t b) {
    return (((uint64_t)k[a] << 32) | a) ^ (((uint64_t)k[b] << 32) | b);
}
inline uint64_t delta(const uint64_t* k, uint32_t a, uint32_t b) {
    uint64_t d = k[a] ^ k[b];
    return d ? d : (uint64_t)(a ^ b);
}

struct MergeCall {
    uint32_t left, right, split;  // inclusive [left, right]; right child starts at split
    bool final;
};

struct Hploc {
    uint32_t n;
    uint32_t radius;
    Node2* nodes;
    std::vector<uint32_t> cluster;
    std::atomic<uint32_t> counter;
    std::atomic<uint32_t> err;
};

// FindNearestNeighbor (BinaryBuilder.cu:126-163), lane by lane: shuffle
// sources wrap modulo 32, candidate areas are compared as uint32 bit
// patterns with strict <.
void find_nn(uint32_t num, const Box* cb, uint32_t radius, uint32_t* nn) {
    uint32_t ma[32], mi[32];
    for (int l = 0; l < 32; ++l) ma[l] = mi[l] = kInvalid;
    for (uint32_t r = 1; r <= radius; ++r) {
        uint32_t ar[32], nna[32], nni[32];
        for (uint32_t l = 0; l < 32; ++l) {
            uint32_t j = l + r;
            ar[l] = kInvalid;
            if (j < num) {
                Box nb = cb[j & 31];
                grow(nb, cb[l]);
                ar[l] = fbits(area(nb));
                if (ar[l] < ma[l]) {
                    ma[l] = ar[l];
                    mi[l] = j;
                }
            }
        }
        for (uint32_t l = 0; l < 32; ++l) {
            uint32_t s = (l + r) & 31;
            nna[l] = ma[s];
            nni[l] = mi[s];
            if (ar[l] < nna[l]) {
                nna[l] = ar[l];
                nni[l] = l;
            }
        }
        for (uint32_t l = 0; l < 32; ++l) {
            uint32_t s = (l - r) & 31;
            ma[l] = nna[s];
            mi[l] = nni[s];
        }
    }
    for (int l = 0; l < 32; ++l) nn[l] = mi[l];
}

// __fns(mask, 0, k): bit position of the k-th set bit (k >= 1), or -1.
inline int fns(uint32_t mask, uint32_t k) {
    for (int b = 0; b < 32; ++b)
        if ((mask >> b) & 1u) {
            if (--k == 0) return b;
        }
    return -1;
}

// MergeClustersCreateBVH2Node (BinaryBuilder.cu:71-124).
uint32_t merge_clusters(Hploc& st, uint32_t num, const uint32_t* nn, uint32_t* cid, Box* cb) {
    uint32_t mask = 0;
    bool mutual[32], mrg[32];
    for (uint32_t l = 0; l < 32; ++l) {
        uint32_t nnn = nn[nn[l] & 31];
        mutual[l] = l < num && l == nnn;
        mrg[l] = mutual[l] && l < nn[l];
        if (mrg[l]) mask |= 1u << l;
    }
    uint32_t cnt = (uint32_t)__builtin_popcount(mask);
    uint32_t base = st.counter.fetch_add(cnt);
    uint32_t ncid[32];
    Box nbb[32];
    for (uint32_t l = 0; l < 32; ++l) {
        ncid[l] = cid[nn[l] & 31];
        nbb[l] = cb[nn[l] & 31];
    }
    for (uint32_t l = 0; l < 32; ++l) {
        if (!mrg[l]) continue;
        uint32_t rel = (uint32_t)__builtin_popcount(mask & ((1u << l) - 1u));
        grow(cb[l], nbb[l]);
        uint32_t idx = base + rel;
        if (idx >= 2 * st.n - 1) {
            st.err.fetch_or(2);
            continue;
        }
        st.nodes[idx].b = cb[l];
        st.nodes[idx].left = cid[l];
        st.nodes[idx].right = ncid[l];
        cid[l] = idx;
    }
    uint32_t valid = 0;
    for (uint32_t l = 0; l < 32; ++l)
        if (mrg[l] || !mutual[l]) valid |= 1u << l;
    uint32_t c2[32];
    Box b2[32];
    for (uint32_t l = 0; l < 32; ++l) {
        int sh = fns(valid, l + 1);
        uint32_t s = sh < 0 ? 31u : (uint32_t)sh;
        c2[l] = sh < 0 ? kInvalid : cid[s];
        b2[l] = cb[s];
    }
    std::memcpy(cid, c2, sizeof(c2));
    std::memcpy(cb, b2, sizeof(b2));
    return num - cnt;
}

// PlocMerge with LoadIndices / StoreIndices (BinaryBuilder.cu:42-69,165-197).
void ploc_merge(Hploc& st, const MergeCall& c) {
    const uint32_t kThreshold = 16;  // MERGING_THRESHOLD, BinaryBuilder.cu:10
    uint32_t lStart = c.left, rEnd = c.right + 1, lEnd = c.split, rStart = c.split;
    uint32_t cid[32];
    for (int l = 0; l < 32; ++l) cid[l] = kInvalid;
    auto load = [&](uint32_t start, uint32_t end, uint32_t offset) {
        uint32_t lim = std::min(end - start, kThreshold), cnt = 0;
        for (uint32_t l = 0; l < 32; ++l) {
            uint32_t idx = l - offset;
            bool valid = idx < lim;
            if (valid) cid[l] = st.cluster[start + idx];
            if (valid && cid[l] != kInvalid) ++cnt;
        }
        return cnt;
    };
    uint32_t numLeft = load(lStart, lEnd, 0);
    uint32_t numRight = load(rStart, rEnd, numLeft);
    uint32_t num = numLeft + numRight;
    Box cb[32];
    std::memset(cb, 0, sizeof(cb));
    for (uint32_t l = 0; l < num; ++l) {
        if (cid[l] == kInvalid || cid[l] >= 2 * st.n - 1) {
            st.err.fetch_or(1);
            return;
        }
        cb[l] = st.nodes[cid[l]].b;
    }
    uint32_t threshold = c.final ? 1 : kThreshold;
    while (num > threshold) {
        uint32_t nn[32];
        find_nn(num, cb, st.radius, nn);
        num = merge_clusters(st, num, nn, cid, cb);
    }
    for (uint32_t l = 0; l < numLeft + numRight; ++l) st.cluster[lStart + l] = cid[l];
}

// BuildBVH2Kernel climb (BinaryBuilder.cu:200-273) with FindParentId
// (:30-40), simulated leaf by leaf; any order is a legal GPU schedule.  The
// PLOC merges it triggers are recorded in a valid bottom-up order.
template <class K>
void lbvh_climb(const K* keys, uint32_t n, std::vector<MergeCall>& calls) {
    std::vector<uint32_t> parent(n, kInvalid);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t left = i, right = i, split = 0;
        while (true) {
            uint32_t prev;
            bool go_right = left == 0 || (right != n - 1 && delta(keys, right, right + 1) < delta(keys, left - 1, left));
            if (go_right) {
                prev = parent[right];
                parent[right] = left;
                if (prev != kInvalid) {
                    split = right + 1;
                    right = prev;
                }
            } else {
                prev = parent[left - 1];
                parent[left - 1] = right;
                if (prev != kInvalid) {
                    split = left;
                    left = prev;
                }
            }
            if (prev == kInvalid) break;
            uint32_t size = right - left + 1;
            bool final = size == n;
            if (size > 16 || final) calls.push_back({left, right, split, final});
        }
    }
}

template <class K>
int hploc(const K* keys, const uint32_t* perm, uint32_t n, uint32_t radius, Node2* nodes, uint32_t* root) {
    Hploc st;
    st.n = n;
    st.radius = radius;
    st.nodes = nodes;
    st.cluster.assign(perm, perm + n);
    st.counter = n;
    st.err = 0;
    std::vector<MergeCall> calls;
    lbvh_climb(keys, n, calls);
    // Merges whose range lies inside one chunk of the leaf range only depend
    // on merges inside that chunk; the rest run afterwards in list order.
    int nt = std::max(1, std::min(threads(), (int)(n / 4096)));
    std::vector<uint32_t> cut((size_t)nt + 1);
    for (int t = 0; t <= nt; ++t) cut[t] = (uint32_t)(((uint64_t)n * t) / nt);
    std::vector<std::vector<uint32_t>> inside((size_t)nt);
    std::vector<uint32_t> crossing;
    for (uint32_t k = 0; k < calls.size(); ++k) {
        const MergeCall& c = calls[k];
        int t = (int)(std::upper_bound(cut.begin(), cut.end(), c.left) - cut.begin()) - 1;
        if (t >= 0 && t < nt && c.right < cut[t + 1])
            inside[t].push_back(k);
        else
            crossing.push_back(k);
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
            for (uint32_t k : inside[t]) ploc_merge(st, calls[k]);
        });
    for (auto& th : pool) th.join();
    for (uint32_t k : crossing) ploc_merge(st, calls[k]);
    *root = n == 1 ? 0 : st.cluster[0];
    if (st.counter.load() != 2 * n - 1) st.err.fetch_or(4);
    return (int)st.err.load();
}

// ---------------------------------------------------------- stage 5
constexpr float kQuantStep = 1.0f / 255.0f;  // 1/((1<<NQ)-1), WideConverter.cu:19

inline uint32_t nib(uint32_t x, uint32_t i) { return (x >> (4 * i)) & 0xFu; }
inline void set_nib(uint32_t& x, uint32_t i, uint32_t v) {
    if (i >= 8) return;  // a 32-bit shift by >= 32 clears nothing on the GPU
    x &= ~(0xFu << (4 * i));
    x |= v << (4 * i);
}
inline uint32_t below(uint32_t m, uint32_t i) { return (uint32_t)__builtin_popcount(m & ((1u << i) - 1u)); }

// CeilLog2 / InvPow2 (BuilderUtils.h:335-347).
inline uint32_t ceil_log2(float x) {
    uint32_t ix = fbits(x);
    uint32_t ex = (ix >> 23) & 0xFFu;
    bool pow2 = (ix & ((1u << 23) - 1u)) == 0;
    return ex + (pow2 ? 0u : 1u);
}
inline float inv_pow2(uint8_t eb) { return bitsf((uint32_t)(254 - (int)eb) << 23); }

// GetCost (WideConverter.cu:25-30).
inline float slot_cost(uint32_t s, const float o[3]) {
    float x = ((s >> 2) & 1) ? -o[0] : o[0];
    float y = ((s >> 1) & 1) ? -o[1] : o[1];
    float z = (s & 1) ? -o[2] : o[2];
    return fadd(fadd(x, y), z);
}

// GreedyAssignment (WideConverter.cu:104-153).
uint32_t greedy(const float pc[3], const uint32_t* child, uint32_t n, const Node2* nodes) {
    uint32_t asg = kInvalid;
    for (uint32_t c = 0; c < n; ++c) {
        float best = -3.402823466e+38f;
        uint32_t slot = 0xF;
        const Box& b = nodes[child[c]].b;
        float off[3];
        for (int a = 0; a < 3; ++a) off[a] = fsub(pc[a], fadd(b.mx[a], b.mn[a]));
        for (uint32_t s = 0; s < 8; ++s) {
            if (nib(asg, s) != 0xF) continue;
            float cost = slot_cost(s, off);
            if (cost > best) {
                best = cost;
                slot = s;
            }
        }
        set_nib(asg, slot, c);
    }
    return asg;
}

// AuctionAssignment (WideConverter.cu:50-102) over the cost table of the
// USE_AUCTION branch of BuildBVH8Kernel (:337-358).  The two divisions
// (MAX_COST / maxDim, 1.0f / n) are the fast-math divide on the GPU; they
// are IEEE divisions here.  Unbounded bidding and a bid with no finite
// reward (the reference then writes prices[15]) fall back to the greedy
// assignment, as the GPU kernel does.
constexpr uint32_t kAuctionBidLimit = 4096;

bool auction(const Box& pb, const uint32_t* child, uint32_t n, const Node2* nodes, uint32_t* out) {
    float ext[3];
    for (int a = 0; a < 3; ++a) ext[a] = fsub(pb.mx[a], pb.mn[a]);
    const float max_dim = fmax_gpu(ext[0], fmax_gpu(ext[1], ext[2]));  // fmaxf(float3), CudaMath.h:1132-1135
    float cost_scale = max_dim == 0.0f ? 0.0f : ftz(10.0f / max_dim);   // MAX_COST = 10
    cost_scale = fmul(cost_scale, 0.5f);
    float pc[3], off[8][3];
    for (int a = 0; a < 3; ++a) pc[a] = fadd(pb.mn[a], pb.mx[a]);
    float max_cost = -3.402823466e+38f;
    for (uint32_t c = 0; c < n; ++c) {
        const Box& b = nodes[child[c]].b;
        for (int a = 0; a < 3; ++a) off[c][a] = fmul(fsub(pc[a], fadd(b.mn[a], b.mx[a])), cost_scale);
        const float cost = fadd(fadd(std::fabs(off[c][0]), std::fabs(off[c][1])), std::fabs(off[c][2]));
        if (cost > max_cost) max_cost = cost;
    }
    float prices[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const float threshold = ftz(1.0f / (float)n);
    float epsilon = fmax_gpu(max_cost, threshold);
    uint32_t asg = kInvalid, bids = 0;
    while (epsilon >= threshold) {
        asg = kInvalid;
        uint32_t bidders = 0x76543210u, waiting = n;
        while (waiting > 0) {
            const uint32_t c = nib(bidders, --waiting);
            float win = -3.402823466e+38f, second = -3.402823466e+38f;
            uint32_t slot = 0xF;
            for (uint32_t s = 0; s < 8; ++s) {
                const float reward = fsub(slot_cost(s, off[c]), prices[s]);
                if (reward > win) {
                    second = win;
                    win = reward;
                    slot = s;
                } else if (reward > second) {
                    second = reward;
                }
            }
            if (slot > 7 || ++bids > kAuctionBidLimit) return false;
            prices[slot] = fadd(prices[slot], fadd(fsub(win, second), epsilon));
            const uint32_t prev = nib(asg, slot);
            set_nib(asg, slot, c);
            if (prev != 0xF) set_nib(bidders, waiting++, prev);
        }
        epsilon = fmul(epsilon, 0.125f);  // invTheta, THETA = 8
    }
    *out = asg;
    return true;
}

// CreateBVH8Node (WideConverter.cu:156-206).  Empty slots keep zero
// quantised bytes (the reference leaves them unspecified).
Node8 make_node8(const Box& bounds, const uint32_t* child, uint32_t child_base, uint32_t prim_base, uint32_t asg,
                 uint32_t inner, uint32_t leaf, const Node2* nodes) {
    Node8 nd;
    std::memset(&nd, 0, sizeof(nd));
    float inv[3];
    for (int a = 0; a < 3; ++a) {
        float diag = fsub(bounds.mx[a], bounds.mn[a]);
        nd.p[a] = bounds.mn[a];
        nd.e[a] = (uint8_t)ceil_log2(fmul(diag, kQuantStep));
        inv[a] = inv_pow2(nd.e[a]);
    }
    nd.child_base = child_base;
    nd.prim_base = prim_base;
    for (uint32_t i = 0; i < 8; ++i) {
        uint32_t a = nib(asg, i);
        if (inner & (1u << i)) {
            nd.imask |= (uint8_t)(1u << i);
            nd.meta[i] = (uint8_t)(0x20u | (24u + i));
        } else if (a != 0xF) {
            nd.meta[i] = (uint8_t)(0x20u | below(leaf, i));
        } else {
            continue;
        }
        const Box& cb = nodes[child[a]].b;
        for (int ax = 0; ax < 3; ++ax) {
            nd.qlo[ax][i] = f2u8(std::floor(fmul(fsub(cb.mn[ax], bounds.mn[ax]), inv[ax])));
            nd.qhi[ax][i] = f2u8(std::ceil(fmul(fsub(cb.mx[ax], bounds.mn[ax]), inv[ax])));
        }
    }
    return nd;
}

// One BVH8 node before it is numbered: its children (BVH2 indices), slot
// assignment and inner / leaf slot masks.  This is one work item of
// BuildBVH8Kernel (WideConverter.cu:284-330 the expansion, :332-362 the slot
// assignment); bvh8() and bvh8_levels() both collapse through it.
struct CollapsedNode {
    uint32_t child[8];
    uint32_t asg, inner, leaf;
};

void collapse_node(const Node2* nodes, uint32_t b2, bool use_auction, CollapsedNode& c) {
    const Node2& nd = nodes[b2];
    uint32_t inner = 0, count = 0;
    uint32_t lr[2] = {nd.left, nd.right};
    int msb = 0;
    while (true) {
        float a0 = area(nodes[lr[0]].b), a1 = area(nodes[lr[1]].b);
        uint32_t first = a0 < a1 ? 0 : 1;
        for (uint32_t i = 0; i < 2; ++i) {
            uint32_t idx = i == 0 ? (uint32_t)msb : count;
            if (nodes[lr[first]].left != kInvalid) inner |= 1u << idx;
            c.child[idx] = lr[first];
            count++;
            first = !first;
        }
        msb = inner ? 31 - __builtin_clz(inner) : -1;
        if (msb < 0 || count == 8) break;
        inner &= ~(1u << msb);
        count--;
        uint32_t ni = c.child[msb];
        lr[0] = nodes[ni].left;
        lr[1] = nodes[ni].right;
    }
    float pc[3];
    for (int a = 0; a < 3; ++a) pc[a] = fadd(nd.b.mn[a], nd.b.mx[a]);
    uint32_t asg = 0;
    if (!use_auction || !auction(nd.b, c.child, count, nodes, &asg)) asg = greedy(pc, c.child, count, nodes);
    c.asg = asg;
    c.inner = c.leaf = 0;
    for (uint32_t i = 0; i < 8; ++i) {
        if (nib(asg, i) == 0xF) continue;
        uint32_t bit = (inner >> nib(asg, i)) & 1u;
        c.inner |= bit << i;
        c.leaf |= (bit ^ 1u) << i;
    }
}

// BuildBVH8Kernel (WideConverter.cu:225-414), with the work slots processed
// in increasing order (every slot is written by a parent in a lower slot).
int bvh8(const Node2* nodes, uint32_t n, uint32_t root, Node8* out, uint32_t cap, uint32_t* prim_idx,
         uint32_t* node_count, uint32_t* leaf_count, bool use_auction = false) {
    if (n == 1) {  // CreateBVH8SingleLeaf (WideConverter.cu:209-222)
        uint32_t child[8] = {0};
        out[0] = make_node8(nodes[0].b, child, 0, 0, 0xFFFFFFF0u, 0, 1, nodes);
        prim_idx[0] = 0;
        *node_count = 1;
        *leaf_count = 1;
        return 0;
    }
    std::vector<uint64_t> pairs(n, ~0ull);
    pairs[0] = (uint64_t)root << 32;
    uint32_t node_ctr = 1, leaf_ctr = 0, work_alloc = 1;
    int err = 0;
    for (uint32_t w = 0; w < n; ++w) {
        while (true) {
            uint64_t pr = pairs[w];
            uint32_t b2 = (uint32_t)(pr >> 32), b8 = (uint32_t)pr;
            if (b2 == kInvalid) return err | 1;
            const Node2& nd = nodes[b2];
            if (nd.left == kInvalid) {
                if (b8 >= n) return err | 2;
                prim_idx[b8] = nd.right;
                break;
            }
            CollapsedNode cn;
            collapse_node(nodes, b2, use_auction, cn);
            const uint32_t* child = cn.child;
            const uint32_t asg = cn.asg, inner = cn.inner, leaf = cn.leaf;
            const uint32_t count = (uint32_t)__builtin_popcount(inner | leaf);
            uint32_t inner_count = (uint32_t)__builtin_popcount(inner);
            uint32_t lc = count - inner_count;
            uint32_t child_base = node_ctr;
            node_ctr += inner_count;
            uint32_t work_base = work_alloc;
            work_alloc += count - 1;
            uint32_t prim_base = 0;
            if (lc > 0) {
                prim_base = leaf_ctr;
                leaf_ctr += lc;
            }
            if (node_ctr > cap || work_alloc > n) return err | 4;
            for (uint32_t i = 0; i < 8; ++i) {
                if (nib(asg, i) == 0xF) continue;
                uint64_t pr2 = (uint64_t)child[nib(asg, i)] << 32;
                if (inner & (1u << i))
                    pr2 |= child_base + below(inner, i);
                else
                    pr2 |= prim_base + below(leaf, i);
                uint32_t c = below(inner | leaf, i);
                uint32_t idx = c == 0 ? w : work_base + c - 1;
                pairs[idx] = pr2;
            }
            out[b8] = make_node8(nd.b, child, child_base, prim_base, asg, inner, leaf, nodes);
        }
    }
    *node_count = node_ctr;
    *leaf_count = leaf_ctr;
    return err;
}

// The same collapse level by level, for the timed CPU baseline: the nodes of
// one BVH8 level are collapsed in parallel, numbered by a prefix sum over the
// level, and written in parallel.  Nodes and primitive slots are numbered
// breadth-first instead of in work-slot order, so the tree equals bvh8()'s
// up to that numbering (canonically identical).
int bvh8_levels(const Node2* nodes, uint32_t n, uint32_t root, Node8* out, uint32_t cap, uint32_t* prim_idx,
                uint32_t* node_count, uint32_t* leaf_count, bool use_auction = false) {
    if (n == 1) return bvh8(nodes, n, root, out, cap, prim_idx, node_count, leaf_count, use_auction);
    std::vector<uint32_t> level = {root};  // BVH2 node of each BVH8 node of the level
    uint32_t level_first = 0;              // BVH8 index of the level's first node
    uint32_t node_ctr = 1, leaf_ctr = 0;
    std::vector<CollapsedNode> col;
    std::vector<uint32_t> cbase, pbase, next;
    while (!level.empty()) {
        const size_t m = level.size();
        col.resize(m);
        parallel_for(m, [&](size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) collapse_node(nodes, level[k], use_auction, col[k]);
        }, 1024);
        cbase.resize(m);
        pbase.resize(m);
        const uint32_t next_first = node_ctr;
        for (size_t k = 0; k < m; ++k) {
            const uint32_t ic = (uint32_t)__builtin_popcount(col[k].inner);
            const uint32_t lc = (uint32_t)__builtin_popcount(col[k].leaf);
            cbase[k] = node_ctr;
            node_ctr += ic;
            pbase[k] = lc ? leaf_ctr : 0;
            leaf_ctr += lc;
        }
        if (node_ctr > cap) return 4;
        if (leaf_ctr > n) return 2;
        next.assign(node_ctr - next_first, kInvalid);
        parallel_for(m, [&](size_t b, size_t e) {
            for (size_t k = b; k < e; ++k) {
                const CollapsedNode& c = col[k];
                out[level_first + k] =
                    make_node8(nodes[level[k]].b, c.child, cbase[k], pbase[k], c.asg, c.inner, c.leaf, nodes);
                for (uint32_t i = 0; i < 8; ++i) {
                    if (nib(c.asg, i) == 0xF) continue;
                    const uint32_t ch = c.child[nib(c.asg, i)];
                    if (c.inner & (1u << i))
                        next[cbase[k] + below(c.inner, i) - next_first] = ch;
                    else
                        prim_idx[pbase[k] + below(c.leaf, i)] = nodes[ch].right;
                }
            }
        }, 1024);
        level.swap(next);
        level_first = next_first;
    }
    *node_count = node_ctr;
    *leaf_count = leaf_ctr;
    return 0;
}

// ---------------------------------------------------------- cost
// ComputeBVH2CostKernel (Eval.cu:12-33): internal C_T=3, leaf C_I=2.
double bvh2_cost(const Node2* nodes, uint32_t count, const Box& root) {
    double ra = area(root), s = 0.0;
    for (uint32_t i = 0; i < count; ++i) {
        double m = (double)area(nodes[i].b) / ra;
        s += (nodes[i].left != kInvalid ? 3.0 : 2.0) * m;
    }
    return s;
}
// ComputeBVH8CostKernel (Eval.cu:36-80): children only; internal C_I=2,
// leaf C_T=3; boxes decoded as p + 2^(e-127) * q.
double bvh8_cost(const Node8* nodes, uint32_t count, const Box& root) {
    double ra = area(root), s = 0.0;
    for (uint32_t i = 0; i < count; ++i) {
        const Node8& nd = nodes[i];
        for (int c = 0; c < 8; ++c) {
            if (!nd.meta[c]) continue;
            bool internal = (nd.meta[c] & 0x1F) >= 24;
            Box b;
            for (int a = 0; a < 3; ++a) {
                float sc = bitsf((uint32_t)nd.e[a] << 23);
                b.mn[a] = ffma(sc, (float)nd.qlo[a][c], nd.p[a]);
                b.mx[a] = ffma(sc, (float)nd.qhi[a][c], nd.p[a]);
            }
            s += (internal ? 2.0 : 3.0) * ((double)area(b) / ra);
        }
    }
    return s;
}

bool same_box(const Box& a, const Box& b) { return std::memcmp(&a, &b, sizeof(Box)) == 0; }

}  // namespace

// =================================================================== C API
extern "C" {

void orc_set_threads(int t) { g_threads = t; }
void orc_set_level_collapse(int on) { g_level_collapse = on != 0; }
int orc_get_threads(void) { return threads(); }
void orc_set_area_form(int f) { g_area_form = f; }
int orc_get_area_form(void) { return g_area_form; }
void orc_set_u8_mode(int m) { g_u8_mode = m; }
int orc_get_u8_mode(void) { return g_u8_mode; }
void orc_set_min_zero_mode(int m) { g_min_zero = m; }

float orc_area(const float* box6) {
    Box b;
    std::memcpy(&b, box6, sizeof(Box));
    return area(b);
}
float orc_fmin(float a, float b) { return fmin_gpu(a, b); }
float orc_fmax(float a, float b) { return fmax_gpu(a, b); }
uint8_t orc_f2u8(float x) { return f2u8(x); }

// Lane-by-lane FindNearestNeighbor for one warp: boxes32 holds 32 boxes
// (6 floats each), the first `num` active.
// The auction slot assignment of one BVH8 node: the parent's box and
// `count` (1..8) child boxes, 6 floats each.  Returns 1 and the nibble-packed
// assignment, or 0 where the oracle falls back to the greedy assignment
// (bid limit, or a bid with no finite reward).
int orc_auction(const float* parent6, const float* child6, uint32_t count, uint32_t* out) {
    if (count == 0 || count > 8) return 0;
    Node2 nodes[8];
    uint32_t child[8];
    for (uint32_t c = 0; c < count; ++c) {
        for (int a = 0; a < 3; ++a) {
            nodes[c].b.mn[a] = child6[6 * c + a];
            nodes[c].b.mx[a] = child6[6 * c + 3 + a];
        }
        nodes[c].left = nodes[c].right = kInvalid;
        child[c] = c;
    }
    Box pb;
    for (int a = 0; a < 3; ++a) {
        pb.mn[a] = parent6[a];
        pb.mx[a] = parent6[3 + a];
    }
    return auction(pb, child, count, nodes, out) ? 1 : 0;
}

void orc_find_nn(uint32_t num, const float* boxes32, uint32_t radius, uint32_t* nn32) {
    Box cb[32];
    std::memcpy(cb, boxes32, sizeof(cb));
    find_nn(num, cb, radius, nn32);
}

void orc_scene_bounds(const float* prims, int prim_type, uint32_t n, void* leaves, float* scene6) {
    Box s;
    scene_bounds(prims, prim_type, n, (Node2*)leaves, &s);
    std::memcpy(scene6, &s, sizeof(Box));
}

void orc_morton(const void* leaves, uint32_t n, const float* scene6, int key_bits, void* keys, uint32_t* cluster) {
    Box s;
    std::memcpy(&s, scene6, sizeof(Box));
    morton((const Node2*)leaves, n, s, key_bits, keys, cluster);
}

// Per-axis quantised coordinates and the float products they truncate, for
// the boundary-tolerance check of the Morton stage.
void orc_morton_quantised(const void* leaves, uint32_t n, const float* scene6, int key_bits, uint32_t* q3,
                          float* prod3) {
    Box s;
    std::memcpy(&s, scene6, sizeof(Box));
    float scale = key_bits == 30 ? 1023.0f : 2097151.0f;
    const Node2* lv = (const Node2*)leaves;
    parallel_for(n, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) quantise(lv[i].b, s, scale, q3 + 3 * i, prod3 + 3 * i);
    });
}

void orc_radix_sort(int key_bytes, const void* keys_in, const uint32_t* vals_in, uint32_t n, uint32_t begin_bit,
                    uint32_t end_bit, void* keys_out, uint32_t* vals_out) {
    if (key_bytes == 4)
        radix_sort((const uint32_t*)keys_in, vals_in, n, begin_bit, end_bit, (uint32_t*)keys_out, vals_out);
    else
        radix_sort((const uint64_t*)keys_in, vals_in, n, begin_bit, end_bit, (uint64_t*)keys_out, vals_out);
}

// std::stable_sort by (key >> begin) restricted to [begin, end): the
// definition the radix sort is checked against.
void orc_stable_sort(int key_bytes, const void* keys_in, uint32_t n, uint32_t begin_bit, uint32_t end_bit,
                     void* keys_out, uint32_t* vals_out) {
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    uint32_t w = end_bit - begin_bit;
    if (key_bytes == 4) {
        const uint32_t* k = (const uint32_t*)keys_in;
        uint64_t m = w >= 64 ? ~0ull : ((1ull << w) - 1);
        std::stable_sort(idx.begin(), idx.end(),
                         [&](uint32_t a, uint32_t b) { return ((k[a] >> begin_bit) & m) < ((k[b] >> begin_bit) & m); });
        for (uint32_t i = 0; i < n; ++i) ((uint32_t*)keys_out)[i] = k[idx[i]];
    } else {
        const uint64_t* k = (const uint64_t*)keys_in;
        uint64_t m = w >= 64 ? ~0ull : ((1ull << w) - 1);
        std::stable_sort(idx.begin(), idx.end(),
                         [&](uint32_t a, uint32_t b) { return ((k[a] >> begin_bit) & m) < ((k[b] >> begin_bit) & m); });
        for (uint32_t i = 0; i < n; ++i) ((uint64_t*)keys_out)[i] = k[idx[i]];
    }
    std::memcpy(vals_out, idx.data(), sizeof(uint32_t) * n);
}

// nodes: 2n-1 entries with leaves [0,n) already filled.  Returns 0 or an
// error bitmask (1: invalid cluster loaded, 2: node overflow, 4: count).
int orc_hploc(int key_bytes, const void* sorted_keys, const uint32_t* perm, uint32_t n, uint32_t radius,
              void* nodes, uint32_t* root) {
    if (n == 0) return 8;
    if (key_bytes == 4) return hploc((const uint32_t*)sorted_keys, perm, n, radius, (Node2*)nodes, root);
    return hploc((const uint64_t*)sorted_keys, perm, n, radius, (Node2*)nodes, root);
}

int orc_bvh8(const void* bvh2_nodes, uint32_t n, uint32_t root, void* bvh8_nodes, uint32_t cap, uint32_t* prim_idx,
             uint32_t* node_count, uint32_t* leaf_count) {
    return bvh8((const Node2*)bvh2_nodes, n, root, (Node8*)bvh8_nodes, cap, prim_idx, node_count, leaf_count);
}
// flags: 1 = auction slot assignment (NXB_BUILD_AUCTION); 2 = the
// level-parallel collapse (breadth-first numbering).
int orc_bvh8_ex(const void* bvh2_nodes, uint32_t n, uint32_t root, void* bvh8_nodes, uint32_t cap,
                uint32_t* prim_idx, uint32_t* node_count, uint32_t* leaf_count, uint32_t flags) {
    if (flags & 2u)
        return bvh8_levels((const Node2*)bvh2_nodes, n, root, (Node8*)bvh8_nodes, cap, prim_idx, node_count,
                           leaf_count, (flags & 1u) != 0);
    return bvh8((const Node2*)bvh2_nodes, n, root, (Node8*)bvh8_nodes, cap, prim_idx, node_count, leaf_count,
                (flags & 1u) != 0);
}

double orc_bvh2_cost(const void* nodes, uint32_t count, const float* root6) {
    Box r;
    std::memcpy(&r, root6, sizeof(Box));
    return bvh2_cost((const Node2*)nodes, count, r);
}
double orc_bvh8_cost(const void* nodes, uint32_t count, const float* root6) {
    Box r;
    std::memcpy(&r, root6, sizeof(Box));
    return bvh8_cost((const Node8*)nodes, count, r);
}

// Exhaustive BVH2 check from `root`.  report[0..7] = nodes visited, leaves,
// duplicate prims, missing prims, parents != union of children, children
// not inside parent, bad child index, max depth.  Returns the error total.
uint64_t orc_validate_bvh2(const void* nodes_v, uint32_t n, uint32_t root, uint64_t* report) {
    const Node2* nodes = (const Node2*)nodes_v;
    uint64_t rep[8] = {0};
    std::vector<uint8_t> seen(n, 0);
    std::vector<std::pair<uint32_t, uint32_t>> stack;
    uint32_t total = 2 * n - 1;
    stack.push_back({root, 0});
    while (!stack.empty()) {
        auto [i, d] = stack.back();
        stack.pop_back();
        if (i >= total) {
            rep[6]++;
            continue;
        }
        if (rep[0] == total) {  // more visits than nodes: a shared subtree or a cycle; stop the walk
            rep[0]++;
            break;
        }
        rep[0]++;
        rep[7] = std::max<uint64_t>(rep[7], d);
        const Node2& nd = nodes[i];
        if (nd.left == kInvalid) {
            rep[1]++;
            if (nd.right >= n)
                rep[6]++;
            else if (seen[nd.right]++)
                rep[2]++;
            continue;
        }
        if (nd.left >= total || nd.right >= total) {
            rep[6]++;
            continue;
        }
        Box u = nodes[nd.left].b;
        grow(u, nodes[nd.right].b);
        if (!same_box(u, nd.b)) rep[4]++;
        for (uint32_t c : {nd.left, nd.right}) {
            const Box& cb = nodes[c].b;
            for (int a = 0; a < 3; ++a)
                if (!(cb.mn[a] >= nd.b.mn[a] && cb.mx[a] <= nd.b.mx[a])) {
                    rep[5]++;
                    break;
                }
        }
        stack.push_back({nd.right, d + 1});
        stack.push_back({nd.left, d + 1});
    }
    for (uint32_t p = 0; p < n; ++p)
        if (!seen[p]) rep[3]++;
    if (report) std::memcpy(report, rep, sizeof(rep));
    return rep[2] + rep[3] + rep[4] + rep[5] + rep[6] + (rep[0] != total) + (rep[1] != n);
}

// Exhaustive BVH8 check.  leaves = the BVH2 leaves [0,n) (exact prim
// boxes).  report[0..9] = nodes visited, leaves, duplicate prims, missing
// prims, bad child index, quantised lo not conservative, quantised hi not
// conservative, slots used, max depth, meta errors.  Conservativeness is
// judged in exact arithmetic: p + 2^(e-127)*q against the exact union of
// the subtree's primitive boxes.
uint64_t orc_validate_bvh8(const void* nodes_v, uint32_t node_count, const uint32_t* prim_idx, uint32_t n,
                           const void* leaves_v, uint64_t* report) {
    const Node8* nodes = (const Node8*)nodes_v;
    const Node2* leaves = (const Node2*)leaves_v;
    uint64_t rep[10] = {0};
    std::vector<uint8_t> seen(n, 0);
    std::vector<uint32_t> order;
    std::vector<uint32_t> depth(node_count, 0);
    std::vector<uint8_t> visited(node_count, 0);
    order.reserve(node_count);
    std::vector<uint32_t> stack = {0};
    while (!stack.empty()) {
        uint32_t i = stack.back();
        stack.pop_back();
        if (i >= node_count || visited[i]) {
            rep[4]++;
            continue;
        }
        visited[i] = 1;
        order.push_back(i);
        rep[0]++;
        rep[8] = std::max<uint64_t>(rep[8], depth[i]);
        const Node8& nd = nodes[i];
        uint32_t leafmask = 0;
        for (uint32_t s = 0; s < 8; ++s)
            if (nd.meta[s] && !((nd.imask >> s) & 1u)) leafmask |= 1u << s;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!nd.meta[s]) {
                if ((nd.imask >> s) & 1u) rep[9]++;
                continue;
            }
            rep[7]++;
            if ((nd.imask >> s) & 1u) {
                if (nd.meta[s] != (uint8_t)(0x20u | (24u + s))) rep[9]++;
                uint32_t c = nd.child_base + below(nd.imask, s);
                if (c >= node_count) {
                    rep[4]++;
                    continue;
                }
                depth[c] = depth[i] + 1;
                stack.push_back(c);
            } else {
                if (nd.meta[s] != (uint8_t)(0x20u | below(leafmask, s))) rep[9]++;
                rep[1]++;
                uint32_t li = nd.prim_base + (nd.meta[s] & 0x1Fu);
                if (li >= n || prim_idx[li] >= n) {
                    rep[4]++;
                    continue;
                }
                if (seen[prim_idx[li]]++) rep[2]++;
            }
        }
    }
    for (uint32_t p = 0; p < n; ++p)
        if (!seen[p]) rep[3]++;
    // exact subtree boxes, children before parents
    std::vector<Box> sub(node_count);
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        uint32_t i = *it;
        const Node8& nd = nodes[i];
        Box acc;
        for (int a = 0; a < 3; ++a) {
            acc.mn[a] = 3.402823466e+38f;
            acc.mx[a] = -3.402823466e+38f;
        }
        uint32_t leafmask = 0;
        for (uint32_t s = 0; s < 8; ++s)
            if (nd.meta[s] && !((nd.imask >> s) & 1u)) leafmask |= 1u << s;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!nd.meta[s]) continue;
            Box cb;
            if ((nd.imask >> s) & 1u) {
                uint32_t c = nd.child_base + below(nd.imask, s);
                if (c >= node_count) continue;
                cb = sub[c];
            } else {
                uint32_t li = nd.prim_base + (nd.meta[s] & 0x1Fu);
                if (li >= n || prim_idx[li] >= n) continue;
                cb = leaves[prim_idx[li]].b;
            }
            grow(acc, cb);
            for (int a = 0; a < 3; ++a) {
                double sc = std::ldexp(1.0, (int)nd.e[a] - 127);
                double lo = (double)nd.p[a] + sc * nd.qlo[a][s];
                double hi = (double)nd.p[a] + sc * nd.qhi[a][s];
                if (lo > (double)cb.mn[a]) rep[5]++;
                if (hi < (double)cb.mx[a]) rep[6]++;
            }
        }
        sub[i] = acc;
    }
    if (report) std::memcpy(report, rep, sizeof(rep));
    return rep[2] + rep[3] + rep[4] + rep[9] + (rep[0] != node_count) + (rep[1] != n);
}

// Canonical comparison of two BVH2s (DFS from each root, children in
// order): topology, every box bit for bit and every leaf's primitive.
// Returns 0 when identical; else the 1-based DFS position of the first
// difference.
uint64_t orc_compare_bvh2(const void* a_v, uint32_t a_root, const void* b_v, uint32_t b_root, uint32_t n) {
    const Node2* a = (const Node2*)a_v;
    const Node2* b = (const Node2*)b_v;
    uint32_t total = 2 * n - 1;
    std::vector<std::pair<uint32_t, uint32_t>> stack = {{a_root, b_root}};
    uint64_t pos = 0;
    while (!stack.empty()) {
        auto [ia, ib] = stack.back();
        stack.pop_back();
        ++pos;
        if (ia >= total || ib >= total || pos > total) return pos;  // pos > total: a cycle
        const Node2& x = a[ia];
        const Node2& y = b[ib];
        if (!same_box(x.b, y.b)) return pos;
        bool lx = x.left == kInvalid, ly = y.left == kInvalid;
        if (lx != ly) return pos;
        if (lx) {
            if (x.right != y.right) return pos;
            continue;
        }
        stack.push_back({x.right, y.right});
        stack.push_back({x.left, y.left});
    }
    return pos == total ? 0 : pos + 1;
}

// Canonical comparison of two BVH8s: every byte of every node except the
// child/prim base indices and the quantised bytes of empty slots, children
// followed in slot order, leaves compared by primitive.
uint64_t orc_compare_bvh8(const void* a_v, uint32_t a_count, const uint32_t* a_prim, const void* b_v,
                          uint32_t b_count, const uint32_t* b_prim, uint32_t n) {
    const Node8* a = (const Node8*)a_v;
    const Node8* b = (const Node8*)b_v;
    if (a_count != b_count) return ~0ull;
    std::vector<std::pair<uint32_t, uint32_t>> stack = {{0, 0}};
    uint64_t pos = 0;
    while (!stack.empty()) {
        auto [ia, ib] = stack.back();
        stack.pop_back();
        ++pos;
        if (ia >= a_count || ib >= b_count || pos > a_count) return pos;  // pos > a_count: a cycle
        const Node8& x = a[ia];
        const Node8& y = b[ib];
        if (std::memcmp(x.p, y.p, 12) || std::memcmp(x.e, y.e, 3) || x.imask != y.imask ||
            std::memcmp(x.meta, y.meta, 8))
            return pos;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!x.meta[s]) continue;
            for (int ax = 0; ax < 3; ++ax)
                if (x.qlo[ax][s] != y.qlo[ax][s] || x.qhi[ax][s] != y.qhi[ax][s]) return pos;
            if ((x.imask >> s) & 1u) {
                stack.push_back({x.child_base + below(x.imask, s), y.child_base + below(y.imask, s)});
            } else {
                uint32_t la = x.prim_base + (x.meta[s] & 0x1Fu), lb = y.prim_base + (y.meta[s] & 0x1Fu);
                if (la >= n || lb >= n || a_prim[la] != b_prim[lb]) return pos;
            }
        }
    }
    return pos == a_count ? 0 : pos + 1;
}

// Order-insensitive comparison of two BVH8s: the same nodes (origin,
// exponents) with the same children (quantised boxes, primitives, subtrees)
// in any slot order.  *reordered receives the number of node pairs whose
// slot order differs.  Used where two slot assignments may legitimately
// differ on near-ties (the auction assignment evaluated with the GPU's
// fast-math divide against this file's IEEE divide).
static uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    return h * 1099511628211ull;
}
static bool unordered_hashes(const Node8* nodes, uint32_t count, const uint32_t* prim, uint32_t n,
                             std::vector<uint64_t>& node_h, std::vector<uint64_t>& child_h) {
    // child_h[8*i + s]: hash of slot s of node i (0 for an empty slot)
    node_h.assign(count, 0);
    child_h.assign(8ull * count, 0);
    std::vector<std::pair<uint32_t, bool>> stack = {{0, false}};
    uint64_t pops = 0;
    while (!stack.empty()) {
        auto [i, expanded] = stack.back();
        stack.pop_back();
        if (i >= count || ++pops > 2ull * count) return false;  // each node is popped twice; more: a cycle
        const Node8& x = nodes[i];
        if (!expanded) {
            stack.push_back({i, true});
            for (uint32_t s = 0; s < 8; ++s)
                if (x.meta[s] && ((x.imask >> s) & 1u)) stack.push_back({x.child_base + below(x.imask, s), false});
            continue;
        }
        std::vector<uint64_t> kids;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!x.meta[s]) continue;
            uint64_t h = 1469598103934665603ull;
            for (int ax = 0; ax < 3; ++ax) h = mix64(h, ((uint64_t)x.qlo[ax][s] << 8) | x.qhi[ax][s]);
            if ((x.imask >> s) & 1u) {
                const uint32_t c = x.child_base + below(x.imask, s);
                if (c >= count) return false;
                h = mix64(h, node_h[c]);
            } else {
                const uint32_t li = x.prim_base + (x.meta[s] & 0x1Fu);
                if (li >= n) return false;
                h = mix64(h, 0x1000000000ull | prim[li]);
            }
            child_h[8ull * i + s] = h;
            kids.push_back(h);
        }
        std::sort(kids.begin(), kids.end());
        uint64_t h = 1469598103934665603ull;
        uint32_t pe[4];
        std::memcpy(pe, x.p, 12);
        std::memcpy(&pe[3], x.e, 3);
        pe[3] &= 0xFFFFFFu;
        for (int k = 0; k < 4; ++k) h = mix64(h, pe[k]);
        for (uint64_t k : kids) h = mix64(h, k);
        node_h[i] = h;
    }
    return true;
}

uint64_t orc_compare_bvh8_unordered(const void* a_v, uint32_t a_count, const uint32_t* a_prim, const void* b_v,
                                    uint32_t b_count, const uint32_t* b_prim, uint32_t n, uint32_t* reordered) {
    const Node8* a = (const Node8*)a_v;
    const Node8* b = (const Node8*)b_v;
    *reordered = 0;
    if (a_count != b_count || a_count == 0) return ~0ull;
    std::vector<uint64_t> ha, ca, hb, cb;
    if (!unordered_hashes(a, a_count, a_prim, n, ha, ca) || !unordered_hashes(b, b_count, b_prim, n, hb, cb))
        return ~0ull;
    if (ha[0] != hb[0]) return 1;
    // count the node pairs whose slot order differs (walk matched children)
    std::vector<std::pair<uint32_t, uint32_t>> stack = {{0, 0}};
    uint32_t visited = 0;
    while (!stack.empty()) {
        auto [ia, ib] = stack.back();
        stack.pop_back();
        if (++visited > a_count) return 3;  // a cycle
        bool same = true;
        for (uint32_t s = 0; s < 8; ++s) same &= ca[8ull * ia + s] == cb[8ull * ib + s];
        if (!same) ++*reordered;
        std::vector<std::pair<uint64_t, uint32_t>> xa, xb;
        for (uint32_t s = 0; s < 8; ++s) {
            if (a[ia].meta[s] && ((a[ia].imask >> s) & 1u)) xa.push_back({ca[8ull * ia + s], a[ia].child_base + below(a[ia].imask, s)});
            if (b[ib].meta[s] && ((b[ib].imask >> s) & 1u)) xb.push_back({cb[8ull * ib + s], b[ib].child_base + below(b[ib].imask, s)});
        }
        std::sort(xa.begin(), xa.end());
        std::sort(xb.begin(), xb.end());
        if (xa.size() != xb.size()) return 2;
        for (size_t k = 0; k < xa.size(); ++k) {
            if (xa[k].first != xb[k].first) return 2;
            stack.push_back({xa[k].second, xb[k].second});
        }
    }
    return visited == a_count ? 0 : 3;
}

// FNV-1a digests of the canonical DFS serialisations used by
// orc_compare_bvh2 / orc_compare_bvh8, so that golden fixtures can pin a
// whole tree in 8 bytes.
static inline void fnv(uint64_t& h, const void* p, size_t len) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < len; ++i) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
}

uint64_t orc_digest_bvh2(const void* nodes_v, uint32_t root, uint32_t n) {
    const Node2* nodes = (const Node2*)nodes_v;
    uint64_t h = 1469598103934665603ull;
    std::vector<uint32_t> stack = {root};
    uint32_t total = 2 * n - 1, visits = 0;
    while (!stack.empty()) {
        uint32_t i = stack.back();
        stack.pop_back();
        if (i >= total || ++visits > total) return 0;
        const Node2& nd = nodes[i];
        fnv(h, &nd.b, sizeof(Box));
        uint32_t tag = nd.left == kInvalid ? nd.right : kInvalid;
        fnv(h, &tag, 4);
        if (nd.left == kInvalid) continue;
        stack.push_back(nd.right);
        stack.push_back(nd.left);
    }
    return h;
}

uint64_t orc_digest_bvh8(const void* nodes_v, uint32_t count, const uint32_t* prim, uint32_t n) {
    const Node8* nodes = (const Node8*)nodes_v;
    uint64_t h = 1469598103934665603ull;
    std::vector<uint32_t> stack = {0};
    uint32_t visits = 0;
    while (!stack.empty()) {
        uint32_t i = stack.back();
        stack.pop_back();
        if (i >= count || ++visits > count) return 0;
        const Node8& x = nodes[i];
        fnv(h, x.p, 12);
        fnv(h, x.e, 3);
        fnv(h, &x.imask, 1);
        fnv(h, x.meta, 8);
        for (uint32_t s = 0; s < 8; ++s) {
            if (!x.meta[s]) continue;
            for (int ax = 0; ax < 3; ++ax) {
                fnv(h, &x.qlo[ax][s], 1);
                fnv(h, &x.qhi[ax][s], 1);
            }
            if ((x.imask >> s) & 1u) {
                stack.push_back(x.child_base + below(x.imask, s));
            } else {
                uint32_t li = x.prim_base + (x.meta[s] & 0x1Fu);
                if (li >= n) return 0;
                fnv(h, &prim[li], 4);
            }
        }
    }
    return h;
}

// Whole pipeline on the CPU (the timed CPU baseline).  stage_ms[0..4] =
// bounds, Morton, sort, H-PLOC, BVH8 wall milliseconds.  counts[0..2] =
// BVH8 node count, leaf count, BVH2 root.
int orc_build(const float* prims, int prim_type, uint32_t n, int key_bits, uint32_t radius, void* bvh2_nodes,
              void* bvh8_nodes, uint32_t bvh8_cap, uint32_t* prim_idx, uint32_t* counts, double* stage_ms) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    Node2* nodes = (Node2*)bvh2_nodes;
    auto t0 = clk::now();
    Box scene;
    scene_bounds(prims, prim_type, n, nodes, &scene);
    auto t1 = clk::now();
    size_t kb = key_bits == 30 ? 4 : 8;
    std::vector<uint8_t> keys(kb * n), sorted(kb * n);
    morton(nodes, n, scene, key_bits, keys.data(), nullptr);
    auto t2 = clk::now();
    std::vector<uint32_t> perm(n);
    if (kb == 4)
        radix_sort((const uint32_t*)keys.data(), nullptr, n, 2, 32, (uint32_t*)sorted.data(), perm.data());
    else
        radix_sort((const uint64_t*)keys.data(), nullptr, n, 1, 64, (uint64_t*)sorted.data(), perm.data());
    auto t3 = clk::now();
    uint32_t root = 0;
    int err = kb == 4 ? hploc((const uint32_t*)sorted.data(), perm.data(), n, radius, nodes, &root)
                      : hploc((const uint64_t*)sorted.data(), perm.data(), n, radius, nodes, &root);
    auto t4 = clk::now();
    uint32_t nc = 0, lc = 0;
    if (bvh8_nodes)
        err |= (g_level_collapse ? bvh8_levels(nodes, n, root, (Node8*)bvh8_nodes, bvh8_cap, prim_idx, &nc, &lc)
                                 : bvh8(nodes, n, root, (Node8*)bvh8_nodes, bvh8_cap, prim_idx, &nc, &lc))
               << 8;
    auto t5 = clk::now();
    if (counts) {
        counts[0] = nc;
        counts[1] = lc;
        counts[2] = root;
    }
    if (stage_ms) {
        stage_ms[0] = ms(t0, t1);
        stage_ms[1] = ms(t1, t2);
        stage_ms[2] = ms(t2, t3);
        stage_ms[3] = ms(t3, t4);
        stage_ms[4] = ms(t4, t5);
    }
    return err;
}

}  // extern "C"
