// On-device generation of the reference's random digraph, value for value.
//
// The reference draws its matrix on the host (src/graph_generator.cpp:7-46):
// std::mt19937(seed); for every ordered pair i != j in row-major order one
// std::bernoulli_distribution(density) draw, and for an edge one
// std::uniform_int_distribution<int>(wmin, wmax) draw. At n = 32768 that is
// 1.07e9 pairs and ~2.7e9 generator words, ~11 s on one host core. Here:
//
//  1. Word stream. The MT19937 recurrence (Matsumoto & Nishimura, 1998)
//        x[k + 624] = x[k + 397] ^ twist(x[k], x[k + 1]),  output j = temper(x[624 + j])
//     is linear over GF(2), and every bit sequence of it satisfies the
//     characteristic polynomial phi (degree 19937) of the state transition.
//     phi is found once per process by Berlekamp-Massey on 2 * 19937 output
//     bits. The state after J words is sum_i r_i * (x[i], ..., x[i + 623])
//     with r = x^J mod phi (Haramoto et al., 2008, polynomial jump-ahead),
//     so with r_c = (x^L)^c mod phi every chunk of L = 2^25 outputs gets its
//     starting state from the seeded first 20560 words, one CTA per chunk
//     (fw_gen_jump_kernel), and one CTA per chunk then runs the recurrence
//     227 words at a time (fw_gen_words_kernel).
//  2. Parse. A pair takes 2 words (the bernoulli draw: libstdc++'s
//     generate_canonical<double, 53> reads two 32-bit words) plus, for an
//     edge, 1 word and one more per rejection of Lemire's method in
//     uniform_int_distribution. Where pair m starts depends on every earlier
//     draw. The stream is cut into segments of 1024 words; for each segment
//     and each of 4 possible entry offsets the pairs that start inside it are
//     walked (fw_gen_segment_kernel); 256 segments compose into a block
//     (fw_gen_block_kernel); one CTA scans the blocks from word 0
//     (fw_gen_scan_kernel); each block's segments get their entries and first
//     pair numbers (fw_gen_expand_kernel); every segment writes its cells
//     (fw_gen_write_kernel). An entry offset outside the tables (a run of
//     rejections across a segment border) is walked directly.
//  3. Draw decisions in integers. The bernoulli draw fires when
//     X = w1 * 2^32 + w0 is below a threshold X* that the host finds by
//     bisection with std::bernoulli_distribution itself on a scripted
//     engine, so the device needs no FP64 and matches the host library by
//     construction; the weight is Lemire's multiply-shift with the host's
//     rejection threshold, as in libstdc++'s uniform_int_distribution.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <random>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "fw_common.cuh"
#include "fw_internal.h"

namespace fw {
namespace {

// ------------------------------------------------------------ MT19937
constexpr int kMtN = 624, kMtM = 397;
constexpr uint32_t kMtA = 0x9908b0dfu, kUpper = 0x80000000u, kLower = 0x7fffffffu;
constexpr int kMtDeg = 19937;                      // degree of phi
constexpr int kPolyWords = (kMtDeg + 63) / 64;     // 312
constexpr int kBaseWords = kMtDeg + kMtN - 1;      // x[0 .. 19936 + 623]
constexpr int kChunkLog2 = 25;
constexpr uint64_t kChunk = uint64_t(1) << kChunkLog2;  // outputs per generating CTA
constexpr int kStep = kMtN - kMtM;                 // 227 words per step of the recurrence

__host__ __device__ __forceinline__ uint32_t mt_next(uint32_t xk, uint32_t xk1, uint32_t xm) {
    const uint32_t y = (xk & kUpper) | (xk1 & kLower);
    return xm ^ (y >> 1) ^ ((y & 1u) ? kMtA : 0u);
}

__host__ __device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

// x[0 .. count) of the recurrence seeded as std::mt19937(seed).
void mt_sequence(uint32_t seed, std::vector<uint32_t>& x, size_t count) {
    x.assign(count, 0);
    x[0] = seed;
    for (int i = 1; i < kMtN; ++i) x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + (uint32_t)i;
    for (size_t k = kMtN; k < count; ++k) x[k] = mt_next(x[k - kMtN], x[k - kMtN + 1], x[k - kMtN + kMtM]);
}

// ------------------------------------------------------------ GF(2)[x] mod phi
using Poly = std::vector<uint64_t>;  // bit i = coefficient of x^i

inline bool bit_of(const Poly& p, int64_t i) { return (p[(size_t)(i >> 6)] >> (i & 63)) & 1u; }

// dst ^= src << shift (dst large enough).
void xor_shifted(Poly& dst, const Poly& src, int64_t shift) {
    const size_t q = (size_t)(shift >> 6);
    const int s = (int)(shift & 63);
    for (size_t w = 0; w < src.size(); ++w) {
        if (!src[w]) continue;
        dst[q + w] ^= src[w] << s;
        if (s) dst[q + w + 1] ^= src[w] >> (64 - s);
    }
}

// Berlekamp-Massey over GF(2): the shortest connection polynomial C
// (C[0] = 1) with s[n] = sum_{i=1..L} C[i] s[n - i] for n >= L.
Poly berlekamp_massey(const std::vector<uint8_t>& s, int* L_out) {
    const int64_t N = (int64_t)s.size();
    const size_t words = (size_t)(N / 64 + 3);
    Poly rs(words, 0);  // rs[t] = s[N - 1 - t]
    for (int64_t t = 0; t < N; ++t)
        if (s[(size_t)(N - 1 - t)]) rs[(size_t)(t >> 6)] |= uint64_t(1) << (t & 63);
    Poly C(words, 0), B(words, 0), T;
    C[0] = B[0] = 1;
    int64_t L = 0, m = 1;
    for (int64_t n = 0; n < N; ++n) {
        // discrepancy: s[n] + sum_{i=1..L} C[i] * s[n - i], with s[n - i] = rs[N - 1 - n + i]
        const int64_t o = N - 1 - n;
        uint64_t acc = 0;
        for (int64_t q = 0; q <= (L >> 6); ++q) {
            uint64_t c = C[(size_t)q];
            if (q == 0) c &= ~uint64_t(1);
            if (!c) continue;
            const int64_t pos = o + 64 * q;
            const size_t w = (size_t)(pos >> 6);
            const int sh = (int)(pos & 63);
            uint64_t r = rs[w] >> sh;
            if (sh && w + 1 < rs.size()) r |= rs[w + 1] << (64 - sh);
            acc ^= c & r;
        }
        const int d = (int)(s[(size_t)n] ^ (__builtin_popcountll(acc) & 1));
        if (!d) {
            ++m;
        } else if (2 * L <= n) {
            T = C;
            xor_shifted(C, B, m);
            L = n + 1 - L;
            B = T;
            m = 1;
        } else {
            xor_shifted(C, B, m);
            ++m;
        }
    }
    *L_out = (int)L;
    return C;
}

struct Gf2Mod {
    Poly phi;                     // kPolyWords + 1 words, degree kMtDeg
    std::vector<Poly> phi_shift;  // phi << k, k = 0..63, kPolyWords + 1 words each

    // Reduces a product of 2 * kPolyWords words modulo phi.
    void reduce(Poly& p) const {
        for (int64_t d = (int64_t)p.size() * 64 - 1; d >= kMtDeg; --d) {
            if (!bit_of(p, d)) continue;
            const int64_t s = d - kMtDeg;
            const Poly& ps = phi_shift[(size_t)(s & 63)];
            const size_t q = (size_t)(s >> 6);
            for (size_t w = 0; w < ps.size() && q + w < p.size(); ++w) p[q + w] ^= ps[w];
        }
        p.resize(kPolyWords);
    }

    Poly mul(const Poly& a, const Poly& b) const {
        std::vector<Poly> bs(64, Poly(kPolyWords + 1, 0));
        for (int k = 0; k < 64; ++k)
            for (int w = 0; w <= kPolyWords; ++w) {
                const uint64_t lo = w < kPolyWords ? b[(size_t)w] : 0;
                const uint64_t hi = (w > 0 && k) ? b[(size_t)w - 1] >> (64 - k) : 0;
                bs[(size_t)k][(size_t)w] = (lo << k) | hi;
            }
        Poly p(2 * kPolyWords + 1, 0);
        for (int q = 0; q < kPolyWords; ++q) {
            uint64_t aw = a[(size_t)q];
            while (aw) {
                const int k = __builtin_ctzll(aw);
                aw &= aw - 1;
                const Poly& s = bs[(size_t)k];
                for (int w = 0; w <= kPolyWords; ++w) p[(size_t)(q + w)] ^= s[(size_t)w];
            }
        }
        reduce(p);
        return p;
    }

    Poly sqr(const Poly& a) const {
        auto spread = [](uint32_t v) {
            uint64_t x = v;
            x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
            x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
            x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
            x = (x | (x << 2)) & 0x3333333333333333ull;
            x = (x | (x << 1)) & 0x5555555555555555ull;
            return x;
        };
        Poly p(2 * kPolyWords + 1, 0);
        for (int q = 0; q < kPolyWords; ++q) {
            p[(size_t)(2 * q)] = spread((uint32_t)a[(size_t)q]);
            p[(size_t)(2 * q + 1)] = spread((uint32_t)(a[(size_t)q] >> 32));
        }
        reduce(p);
        return p;
    }
};

// g^e mod phi by square-and-multiply.
Poly g_power(const Gf2Mod& f, const Poly& g, uint64_t e) {
    Poly acc(kPolyWords, 0), base = g;
    acc[0] = 1;
    while (e) {
        if (e & 1) acc = f.mul(acc, base);
        e >>= 1;
        if (e) base = f.sqr(base);
    }
    return acc;
}

// Process-wide jump tables: phi, g = x^kChunk mod phi and r_c = g^c.
struct JumpTables {
    std::mutex mu;
    bool ready = false;
    Gf2Mod field;
    Poly g;
    std::vector<Poly> r;  // r[c] = x^(c * kChunk) mod phi
    std::string error;
};

JumpTables& jump_tables() {
    static JumpTables t;
    return t;
}

// Fills phi and g once; extends r to at least `chunks` entries.
int ensure_jump_tables(size_t chunks) {
    JumpTables& t = jump_tables();
    std::lock_guard<std::mutex> lk(t.mu);
    if (!t.ready) {
        // 2 * deg output bits (bit 0 of consecutive outputs) and 64 more to check.
        const size_t nbits = 2 * kMtDeg + 64;
        std::vector<uint32_t> x;
        mt_sequence(5489u, x, kMtN + nbits);
        std::vector<uint8_t> s(nbits);
        for (size_t k = 0; k < nbits; ++k) s[k] = (uint8_t)(x[kMtN + k] & 1u);
        int L = 0;
        const std::vector<uint8_t> head(s.begin(), s.begin() + 2 * kMtDeg);
        Poly C = berlekamp_massey(head, &L);
        if (L != kMtDeg) return set_error(FW_ERR_INTERNAL, "mt19937 jump: characteristic polynomial has degree " +
                                                               std::to_string(L) + ", expected 19937");
        // the recurrence must also predict the 64 bits it was not fitted on
        for (size_t n = 2 * kMtDeg; n < nbits; ++n) {
            int v = s[n];
            for (int i = 1; i <= L; ++i)
                if (bit_of(C, i)) v ^= s[n - (size_t)i];
            if (v) return set_error(FW_ERR_INTERNAL, "mt19937 jump: characteristic polynomial check failed");
        }
        // phi(x) = x^L C(1/x)
        Poly phi(kPolyWords + 1, 0);
        for (int j = 0; j <= L; ++j)
            if (bit_of(C, L - j)) phi[(size_t)(j >> 6)] |= uint64_t(1) << (j & 63);
        t.field.phi = phi;
        t.field.phi_shift.assign(64, Poly(kPolyWords + 1, 0));
        for (int k = 0; k < 64; ++k) {
            Poly& ps = t.field.phi_shift[(size_t)k];
            for (int w = 0; w <= kPolyWords; ++w) {
                const uint64_t hi = (w > 0 && k) ? phi[(size_t)w - 1] >> (64 - k) : 0;
                ps[(size_t)w] = (phi[(size_t)w] << k) | hi;
            }
        }
        Poly xp(kPolyWords, 0);
        xp[0] = 2;  // x
        for (int i = 0; i < kChunkLog2; ++i) xp = t.field.sqr(xp);
        t.g = xp;
        Poly one(kPolyWords, 0);
        one[0] = 1;
        t.r.push_back(one);
        t.ready = true;
    }
    // r[c] = g^c for the missing c, split over host threads: each thread
    // starts its contiguous range with one exponentiation and walks it with
    // one multiplication per entry.
    const size_t have = t.r.size();
    if (have < chunks) {
        t.r.resize(chunks);
        const size_t todo = chunks - have;
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const size_t workers = std::min<size_t>({(size_t)hw, (size_t)16, (todo + 3) / 4});
        const size_t per = (todo + workers - 1) / workers;
        // A range reads only entries no other thread writes: the ones that
        // existed before this call, else its own start power.
        auto fill = [&](size_t lo, size_t hi) {
            Poly acc = lo - 1 < have ? t.r[lo - 1] : g_power(t.field, t.g, lo - 1);
            for (size_t c = lo; c < hi; ++c) {
                acc = t.field.mul(acc, t.g);
                t.r[c] = acc;
            }
        };
        std::vector<std::thread> pool;
        std::vector<std::pair<size_t, size_t>> here;  // ranges no thread could be started for
        for (size_t w = 1; w < workers; ++w) {
            const size_t lo = have + w * per, hi = std::min(chunks, have + (w + 1) * per);
            if (lo >= hi) continue;
            try {
                pool.emplace_back(fill, lo, hi);
            } catch (const std::system_error&) {
                here.emplace_back(lo, hi);
            }
        }
        fill(have, std::min(chunks, have + per));
        for (const auto& [lo, hi] : here) fill(lo, hi);
        for (auto& th : pool) th.join();
    }
    return FW_OK;
}

// x^e mod phi by square-and-multiply.
Poly x_pow(uint64_t e) {
    JumpTables& t = jump_tables();
    Poly acc(kPolyWords, 0), base(kPolyWords, 0);
    acc[0] = 1;
    base[0] = 2;
    while (e) {
        if (e & 1) acc = t.field.mul(acc, base);
        e >>= 1;
        if (e) base = t.field.sqr(base);
    }
    return acc;
}

// State words (x[J], ..., x[J + 623]) for r = x^J mod phi; x[J]'s low 31 bits
// are not determined (the recurrence never reads them).
void jumped_state(const std::vector<uint32_t>& base, const Poly& r, uint32_t* out) {
    for (int t = 0; t < kMtN; ++t) out[t] = 0;
    for (int i = 0; i < kMtDeg; ++i)
        if (bit_of(r, i))
            for (int t = 0; t < kMtN; ++t) out[t] ^= base[(size_t)(i + t)];
}

// ------------------------------------------------------------ draw parameters
// An engine that returns scripted words, to ask the host library itself how
// it turns words into draws.
struct ScriptedEngine {
    using result_type = std::mt19937::result_type;
    const uint32_t* w;
    int i = 0;
    static constexpr result_type min() { return std::mt19937::min(); }
    static constexpr result_type max() { return std::mt19937::max(); }
    result_type operator()() { return w[i++]; }
};

struct GenParams {
    uint64_t xstar;      // edge iff w1 * 2^32 + w0 < xstar (unless always_edge)
    uint32_t always_edge;
    uint32_t erange;     // wmax - wmin + 1 as uint32; 0 = all 2^32 values
    uint32_t threshold;  // Lemire rejection threshold (2^32 - erange) % erange
    int32_t wmin;
};

bool host_bernoulli(double p, uint64_t X) {
    const uint32_t w[2] = {(uint32_t)X, (uint32_t)(X >> 32)};
    ScriptedEngine e{w};
    std::bernoulli_distribution d(p);
    return d(e);
}

GenParams make_params(double p, int32_t wmin, int32_t wmax) {
    GenParams g{};
    // The draw is monotone in X: find the first X for which it fails.
    if (host_bernoulli(p, ~uint64_t(0))) {
        g.always_edge = 1;
        g.xstar = 0;
    } else {
        uint64_t lo = 0, hi = ~uint64_t(0);  // answer in [lo, hi]
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo) / 2;
            if (host_bernoulli(p, mid))
                lo = mid + 1;
            else
                hi = mid;
        }
        g.xstar = lo;
    }
    const uint64_t range = (uint64_t)((int64_t)wmax - (int64_t)wmin) + 1;
    g.erange = (uint32_t)range;  // 2^32 wraps to 0
    g.threshold = g.erange ? (uint32_t)(0u - g.erange) % g.erange : 0u;
    g.wmin = wmin;
    return g;
}

// ------------------------------------------------------------ parse geometry
constexpr int kSeg = 1024;         // words per segment
constexpr int kEntries = 4;        // tabulated entry offsets per segment
constexpr int kBlockSegs = 256;    // segments per block
constexpr uint32_t kExitWalk = 255;  // table marker: exit offset too large, walk
constexpr int kMaxPairWords = 64;  // a pair longer than this (61 rejections) is an error

struct ParseState {
    const uint32_t* words;
    GenParams g;
    const uint32_t* seg_table;  // [nseg][kEntries]: count << 8 | exit
    uint64_t nseg;
    unsigned* err;
};

// Length in words of the pair whose draw starts at `pos`; *w = its value.
__device__ __forceinline__ uint32_t pair_at(const uint32_t* __restrict__ words, uint64_t pos, const GenParams& g,
                                            int32_t* w, unsigned* err) {
    const uint64_t X = ((uint64_t)words[pos + 1] << 32) | words[pos];
    if (!g.always_edge && X >= g.xstar) {
        *w = kInf;
        return 2;
    }
    if (g.erange == 0) {
        *w = (int32_t)(words[pos + 2] + (uint32_t)g.wmin);
        return 3;
    }
    uint32_t len = 3;
    uint64_t prod = (uint64_t)words[pos + 2] * g.erange;
    uint32_t low = (uint32_t)prod;
    if (low < g.erange) {
        while (low < g.threshold) {
            if (len >= kMaxPairWords) {
                atomicOr(err, 1u);
                break;
            }
            prod = (uint64_t)words[pos + len] * g.erange;
            low = (uint32_t)prod;
            ++len;
        }
    }
    *w = (int32_t)((uint32_t)(prod >> 32) + (uint32_t)g.wmin);
    return len;
}

struct SegStep {
    uint32_t count;  // pairs starting inside the segment
    uint32_t exit;   // entry offset of the next segment
};

__device__ SegStep seg_walk(const ParseState& ps, uint64_t seg, uint32_t entry) {
    uint64_t pos = seg * kSeg + entry;
    const uint64_t end = (seg + 1) * kSeg;
    uint32_t count = 0;
    while (pos < end) {
        int32_t w;
        pos += pair_at(ps.words, pos, ps.g, &w, ps.err);
        ++count;
    }
    return {count, (uint32_t)(pos - end)};
}

__device__ __forceinline__ SegStep seg_step(const ParseState& ps, uint64_t seg, uint32_t entry) {
    if (entry < (uint32_t)kEntries) {
        const uint32_t v = ps.seg_table[seg * kEntries + entry];
        if ((v & 255u) != kExitWalk) return {v >> 8, v & 255u};
    }
    return seg_walk(ps, seg, entry);
}

// ------------------------------------------------------------ kernels
// Chunk c's starting state: word t = XOR of base[i + t] over the set bits i of r_c.
__global__ void __launch_bounds__(640) fw_gen_jump_kernel(const uint32_t* __restrict__ base,
                                                          const uint64_t* __restrict__ polys,
                                                          uint32_t* __restrict__ states) {
    extern __shared__ uint32_t sbase[];  // kBaseWords
    __shared__ uint64_t pr[kPolyWords];
    for (int i = threadIdx.x; i < kBaseWords; i += blockDim.x) sbase[i] = base[i];
    for (int i = threadIdx.x; i < kPolyWords; i += blockDim.x) pr[i] = polys[(size_t)blockIdx.x * kPolyWords + i];
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= kMtN) return;
    uint32_t acc = 0;
    for (int q = 0; q < kPolyWords; ++q) {
        uint64_t w = pr[q];
        while (w) {
            const int b = __ffsll((long long)w) - 1;
            w &= w - 1;
            acc ^= sbase[q * 64 + b + t];
        }
    }
    states[(size_t)blockIdx.x * kMtN + t] = acc;
}

// One CTA per chunk of kChunk outputs: the recurrence on a 1024-word ring in
// shared memory, 227 new words per step, one per thread (they read only words
// of the previous 624, which the step does not overwrite).
constexpr int kGenThreads = 256;
__global__ void __launch_bounds__(kGenThreads) fw_gen_words_kernel(const uint32_t* __restrict__ states,
                                                                   uint32_t* __restrict__ out) {
    __shared__ uint32_t rg[1024];
    const int c = blockIdx.x, t = threadIdx.x;
    for (int i = t; i < kMtN; i += kGenThreads) rg[i] = states[(size_t)c * kMtN + i];
    __syncthreads();
    uint32_t* o = out + (uint64_t)c * kChunk;
    for (uint32_t k0 = 0; k0 < (uint32_t)kChunk; k0 += kStep) {
        const uint32_t k = k0 + (uint32_t)t;
        if (t < kStep && k < (uint32_t)kChunk) {
            const uint32_t xn = mt_next(rg[k & 1023], rg[(k + 1) & 1023], rg[(k + kMtM) & 1023]);
            rg[(k + kMtN) & 1023] = xn;
            o[k] = mt_temper(xn);
        }
        __syncthreads();
    }
}

// Thread per (segment, entry offset): pairs starting inside the segment and
// the exit offset.
__global__ void fw_gen_segment_kernel(ParseState ps, uint32_t* __restrict__ table) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ps.nseg * kEntries) return;
    const SegStep s = seg_walk(ps, t / kEntries, (uint32_t)(t % kEntries));
    table[t] = (s.count << 8) | (s.exit < kExitWalk ? s.exit : kExitWalk);
}

// Thread per (block, entry offset): the block's segments composed.
__global__ void fw_gen_block_kernel(ParseState ps, uint64_t nblk, uint64_t* __restrict__ btab) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nblk * kEntries) return;
    const uint64_t b = t / kEntries;
    uint32_t e = (uint32_t)(t % kEntries);
    uint64_t count = 0;
    const uint64_t g1 = min(ps.nseg, (b + 1) * kBlockSegs);
    for (uint64_t g = b * kBlockSegs; g < g1; ++g) {
        const SegStep s = seg_step(ps, g, e);
        count += s.count;
        e = s.exit;
    }
    btab[t] = (count << 8) | (e < kExitWalk ? e : kExitWalk);
}

// One CTA: entry offset and first pair number of every block, from word 0.
// The block table streams through shared memory so the serial walk of thread
// 0 reads it at shared-memory latency.
constexpr int kScanChunk = 1024;
__global__ void __launch_bounds__(256) fw_gen_scan_kernel(ParseState ps, uint64_t nblk,
                                                          const uint64_t* __restrict__ btab,
                                                          uint32_t* __restrict__ bentry,
                                                          uint64_t* __restrict__ bpair, uint64_t* __restrict__ total) {
    __shared__ uint64_t sm[kScanChunk * kEntries];
    uint32_t e = 0;
    uint64_t pb = 0;
    for (uint64_t b0 = 0; b0 < nblk; b0 += kScanChunk) {
        const uint64_t nb = min((uint64_t)kScanChunk, nblk - b0);
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < nb * kEntries; i += blockDim.x) sm[i] = btab[b0 * kEntries + i];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint64_t b = b0; b < b0 + nb; ++b) {
                bentry[b] = e;
                bpair[b] = pb;
                const uint64_t v = e < (uint32_t)kEntries ? sm[(b - b0) * kEntries + e] : kExitWalk;
                if (e < (uint32_t)kEntries && (v & 255u) != kExitWalk) {
                    pb += v >> 8;
                    e = (uint32_t)(v & 255u);
                } else {
                    const uint64_t g1 = min(ps.nseg, (b + 1) * kBlockSegs);
                    for (uint64_t g = b * kBlockSegs; g < g1; ++g) {
                        const SegStep s = seg_step(ps, g, e);
                        pb += s.count;
                        e = s.exit;
                    }
                }
            }
        }
    }
    if (threadIdx.x == 0) *total = pb;
}

// Thread per block: entry offset and first pair number of each segment.
__global__ void fw_gen_expand_kernel(ParseState ps, uint64_t nblk, const uint32_t* __restrict__ bentry,
                                     const uint64_t* __restrict__ bpair, uint32_t* __restrict__ sentry,
                                     uint64_t* __restrict__ spair) {
    const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    uint32_t e = bentry[b];
    uint64_t pb = bpair[b];
    const uint64_t g1 = min(ps.nseg, (b + 1) * kBlockSegs);
    for (uint64_t g = b * kBlockSegs; g < g1; ++g) {
        sentry[g] = e;
        spair[g] = pb;
        const SegStep s = seg_step(ps, g, e);
        pb += s.count;
        e = s.exit;
    }
}

// Thread per segment: the cells of the pairs that start inside it. Pair m is
// the m-th off-diagonal cell in row-major order.
__global__ void fw_gen_write_kernel(ParseState ps, const uint32_t* __restrict__ sentry,
                                    const uint64_t* __restrict__ spair, uint64_t pairs, int64_t n,
                                    int32_t* __restrict__ D) {
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ps.nseg) return;
    uint64_t m = spair[g];
    if (m >= pairs) return;
    uint64_t pos = g * kSeg + sentry[g];
    const uint64_t end = (g + 1) * kSeg;
    const uint64_t row = (uint64_t)(n - 1);
    uint64_t i = m / row, jj = m - i * row;
    while (pos < end && m < pairs) {
        int32_t w;
        pos += pair_at(ps.words, pos, ps.g, &w, ps.err);
        D[i * (uint64_t)n + jj + (jj >= i ? 1 : 0)] = w;
        ++m;
        if (++jj == row) {
            jj = 0;
            ++i;
        }
    }
}

__global__ void fw_gen_diag_kernel(int32_t* __restrict__ D, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        D[i * n + i] = 0;
}

// Device buffers of one call, released on every return path.
struct GenBuffers {
    cudaStream_t s;
    std::vector<void*> ptrs;
    explicit GenBuffers(cudaStream_t st) : s(st) {}
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), s) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~GenBuffers() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
    }
};

unsigned grid_for(uint64_t threads, unsigned block) { return (unsigned)((threads + block - 1) / block); }

// One attempt with room for `words_needed` generator words; *short_words is
// set when the pairs did not fit.
int generate_attempt(int32_t* d_D, int64_t n, const GenParams& gp, const std::vector<uint32_t>& base,
                     uint64_t words_needed, cudaStream_t s, bool* short_words) {
    *short_words = false;
    const uint64_t pairs = (uint64_t)n * (uint64_t)(n - 1);
    const uint64_t chunks = (words_needed + 2 * kSeg + kMaxPairWords + kChunk - 1) / kChunk;
    if (chunks > 1u << 20) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_generate_graph_device_i32: n too large");
    const uint64_t wgen = chunks * kChunk;
    const uint64_t nseg = (wgen - kSeg - kMaxPairWords) / kSeg;
    const uint64_t nblk = (nseg + kBlockSegs - 1) / kBlockSegs;

    size_t free_b = 0, total_b = 0;
    FW_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const double need = 4.0 * (double)wgen + (4.0 * kEntries + 12.0) * (double)nseg + (double)chunks * 4096.0;
    if (need > 0.9 * (double)free_b)
        return set_error(FW_ERR_NO_MEMORY, "fw_generate_graph_device_i32: needs " + std::to_string((size_t)need) +
                                               " bytes of device memory for n = " + std::to_string(n));
    if (int rc = ensure_jump_tables((size_t)chunks)) return rc;
    std::vector<uint64_t> polys((size_t)chunks * kPolyWords);
    {
        JumpTables& t = jump_tables();
        std::lock_guard<std::mutex> lk(t.mu);
        for (uint64_t c = 0; c < chunks; ++c)
            std::memcpy(&polys[(size_t)c * kPolyWords], t.r[(size_t)c].data(), kPolyWords * sizeof(uint64_t));
    }

    GenBuffers buf(s);
    uint32_t* d_words = buf.get<uint32_t>(wgen);
    uint32_t* d_base = buf.get<uint32_t>(kBaseWords);
    uint64_t* d_polys = buf.get<uint64_t>(polys.size());
    uint32_t* d_states = buf.get<uint32_t>((size_t)chunks * kMtN);
    uint32_t* d_table = buf.get<uint32_t>(nseg * kEntries);
    uint64_t* d_btab = buf.get<uint64_t>(nblk * kEntries);
    uint32_t* d_bentry = buf.get<uint32_t>(nblk);
    uint64_t* d_bpair = buf.get<uint64_t>(nblk);
    uint32_t* d_sentry = buf.get<uint32_t>(nseg);
    uint64_t* d_spair = buf.get<uint64_t>(nseg);
    uint64_t* d_status = buf.get<uint64_t>(2);  // [0] pairs found, [1] error bits
    for (void* p : buf.ptrs)
        if (!p) return set_error(FW_ERR_NO_MEMORY, "fw_generate_graph_device_i32: device allocation failed");
    if (buf.ptrs.size() != 11)
        return set_error(FW_ERR_NO_MEMORY, "fw_generate_graph_device_i32: device allocation failed");

    FW_CUDA_TRY(cudaMemsetAsync(d_status, 0, 2 * sizeof(uint64_t), s));
    FW_CUDA_TRY(cudaMemcpyAsync(d_base, base.data(), kBaseWords * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    FW_CUDA_TRY(
        cudaMemcpyAsync(d_polys, polys.data(), polys.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    const size_t jump_smem = kBaseWords * sizeof(uint32_t);
    FW_CUDA_TRY(cudaFuncSetAttribute(fw_gen_jump_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jump_smem));
    fw_gen_jump_kernel<<<(unsigned)chunks, 640, jump_smem, s>>>(d_base, d_polys, d_states);
    FW_LAUNCH_CHECK("fw_gen_jump_kernel");
    fw_gen_words_kernel<<<(unsigned)chunks, kGenThreads, 0, s>>>(d_states, d_words);
    FW_LAUNCH_CHECK("fw_gen_words_kernel");

    unsigned* d_err = reinterpret_cast<unsigned*>(d_status + 1);
    ParseState ps{d_words, gp, d_table, nseg, d_err};
    fw_gen_segment_kernel<<<grid_for(nseg * kEntries, 256), 256, 0, s>>>(ps, d_table);
    FW_LAUNCH_CHECK("fw_gen_segment_kernel");
    fw_gen_block_kernel<<<grid_for(nblk * kEntries, 128), 128, 0, s>>>(ps, nblk, d_btab);
    FW_LAUNCH_CHECK("fw_gen_block_kernel");
    fw_gen_scan_kernel<<<1, 256, 0, s>>>(ps, nblk, d_btab, d_bentry, d_bpair, d_status);
    FW_LAUNCH_CHECK("fw_gen_scan_kernel");
    fw_gen_expand_kernel<<<grid_for(nblk, 128), 128, 0, s>>>(ps, nblk, d_bentry, d_bpair, d_sentry, d_spair);
    FW_LAUNCH_CHECK("fw_gen_expand_kernel");
    fw_gen_write_kernel<<<grid_for(nseg, 128), 128, 0, s>>>(ps, d_sentry, d_spair, pairs, n, d_D);
    FW_LAUNCH_CHECK("fw_gen_write_kernel");
    fw_gen_diag_kernel<<<grid_for((uint64_t)n, 256) < 1024 ? grid_for((uint64_t)n, 256) : 1024, 256, 0, s>>>(d_D, n);
    FW_LAUNCH_CHECK("fw_gen_diag_kernel");

    uint64_t status[2] = {0, 0};
    FW_CUDA_TRY(cudaMemcpyAsync(status, d_status, sizeof(status), cudaMemcpyDeviceToHost, s));
    FW_CUDA_TRY(cudaStreamSynchronize(s));
    if (status[1] & 0xffffffffu)
        return set_error(FW_ERR_INTERNAL, "fw_generate_graph_device_i32: a weight draw needed more than " +
                                              std::to_string(kMaxPairWords - 3) + " rejections");
    if (status[0] < pairs) *short_words = true;
    return FW_OK;
}

}  // namespace
}  // namespace fw

using namespace fw;

extern "C" {

int fw_generate_graph_device_i32(int32_t* d_D, int64_t n, double density, uint32_t seed, int32_t wmin,
                                 int32_t wmax, fw_stream_t stream) {
    if (d_D == nullptr) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_generate_graph_device_i32: d_D is NULL");
    if (n < 1 || n > 1000000)
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_generate_graph_device_i32: need 1 <= n <= 1000000");
    if (!(density >= 0.0 && density <= 1.0))
        return set_error(FW_ERR_INVALID_ARGUMENT, "fw_generate_graph_device_i32: density must be in [0, 1]");
    if (wmin > wmax) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_generate_graph_device_i32: wmin > wmax");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t sd = seed != 0 ? seed : (uint32_t)std::random_device{}();
    const uint64_t pairs = (uint64_t)n * (uint64_t)(n - 1);
    if (pairs == 0) {
        fw_gen_diag_kernel<<<1, 32, 0, s>>>(d_D, n);
        FW_LAUNCH_CHECK("fw_gen_diag_kernel");
        return FW_OK;
    }
    const GenParams gp = make_params(density, wmin, wmax);
    std::vector<uint32_t> base;
    mt_sequence(sd, base, kBaseWords);
    // Words: 2 per pair, 1 more per edge and per rejection. First try room for
    // the expected count plus a wide margin, then for every pair an edge with
    // twice the expected rejections.
    const double q = gp.erange ? (double)gp.threshold / 4294967296.0 : 0.0;
    const double pe = gp.always_edge ? 1.0 : std::min(1.0, (double)gp.xstar / 18446744073709551616.0);
    const double edges = (double)pairs * pe + 16.0 * std::sqrt((double)pairs) + 1024.0;
    uint64_t words = 2 * pairs + (uint64_t)(edges * (1.0 + 2.0 * q / (1.0 - q))) + 65536;
    for (int attempt = 0; attempt < 2; ++attempt) {
        bool short_words = false;
        if (int rc = generate_attempt(d_D, n, gp, base, words, s, &short_words)) return rc;
        if (!short_words) return FW_OK;
        words = 3 * pairs + (uint64_t)((double)pairs * 4.0 * q / (1.0 - q)) + (uint64_t(1) << 22);
    }
    return set_error(FW_ERR_INTERNAL, "fw_generate_graph_device_i32: generator words ran short");
}

int fw_mt19937_outputs(uint32_t seed, uint64_t skip, int64_t count, uint32_t* h_out) {
    if (h_out == nullptr || count < 0) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_mt19937_outputs: bad arguments");
    // skip = c * kChunk + rem: the chunk table entry r_c (the one the device
    // generator uses for chunk c) times x^rem.
    const uint64_t c = skip / kChunk, rem = skip % kChunk;
    if (c > (1u << 20)) return set_error(FW_ERR_INVALID_ARGUMENT, "fw_mt19937_outputs: skip too large");
    if (int rc = ensure_jump_tables((size_t)c + 1)) return rc;
    std::vector<uint32_t> base;
    mt_sequence(seed, base, kBaseWords);
    Poly r;
    {
        JumpTables& t = jump_tables();
        std::lock_guard<std::mutex> lk(t.mu);
        r = t.field.mul(t.r[(size_t)c], x_pow(rem));
    }
    std::vector<uint32_t> x(kMtN);
    jumped_state(base, r, x.data());
    // x[t] = x_{skip + t}; output skip + j = temper(x_{skip + 624 + j})
    x.resize((size_t)kMtN + (size_t)count);
    for (int64_t j = 0; j < count; ++j) {
        const size_t k = (size_t)j;
        x[k + kMtN] = mt_next(x[k], x[k + 1], x[k + kMtM]);
        h_out[j] = mt_temper(x[k + kMtN]);
    }
    return FW_OK;
}

}  // extern "C"
