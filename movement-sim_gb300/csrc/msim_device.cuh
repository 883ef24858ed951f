// Device-side math of the movement-sim tick: RNGs, the road-graph move step,
// the radius predicate and the spatial tile keys.
//
// Every float operation in the move step and the predicate is an explicit
// round-to-nearest intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn), so
// the compiler cannot contract a multiply and an add into one FMA: results are
// bit-identical to an IEEE binary32 evaluation of the reference GLSL in source
// order (src/sim/shader/random_move.comp).
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace msim {

constexpr uint32_t kHeadToEnd = 0x80000000u;
constexpr uint32_t kHeadRoad = 0x7fffffffu;

// device error word bits
constexpr uint32_t kErrTimeout = 1u;
constexpr uint32_t kErrOob = 2u;

struct DeviceMap {
    const float4* road_pos;   // [R] start.x, start.y, end.x, end.y
    const uint4* road_conn;   // [R] connIndexStart, connCountStart, connIndexEnd, connCountEnd
    const uint32_t* conn;     // [C + 1]; entry C repeats entry C-1
    const float* factor;      // [R] per-road speed factor or nullptr (1.0)
    uint32_t num_roads;
    uint32_t num_conn;        // C
};

// Uniform tile grid over the world [0, W) x [0, H); tile side = 1 / inv_cell.
// Sort key = (Morton code of the tile << ybits) | y band of the entity inside its
// tile (2^ybits bands of equal height), so the entities of a tile are sorted by
// band and a query reads only the bands its box overlaps.
struct TileGrid {
    float inv_cell;
    uint32_t tiles_x;
    uint32_t tiles_y;
    uint32_t bits;   // Morton bits per axis
    float reach;     // radius + rounding margin used to pick candidate tiles
    float radius;
    uint32_t ybits;  // y-band bits below the tile code (0 = none)
    float ybands;    // 2^ybits as a float
    float d2_limit;  // smallest float t with sqrt_rn(t) >= radius (see in_range_fast)
};

// ---- RNG -------------------------------------------------------------------
// xorshift128, random_move.comp:725-736 (uvec4 = x, y, z, w)
__device__ __forceinline__ uint32_t xs128_next(uint4& s) {
    uint32_t t = s.w;
    uint32_t x = s.x;
    s.w = s.z;
    s.z = s.y;
    s.y = x;
    t ^= t << 11;
    t ^= t >> 8;
    s.x = t ^ x ^ (x >> 19);
    return s.x;
}

// PCG-XSH-RR 64/32 (O'Neill 2014); s = {state_lo, state_hi, inc_lo, inc_hi}
__device__ __forceinline__ uint32_t pcg32_next(uint4& s) {
    uint64_t old = ((uint64_t)s.y << 32) | s.x;
    uint64_t inc = ((uint64_t)s.w << 32) | s.z;
    uint64_t nxt = old * 6364136223846793005ULL + inc;
    s.x = (uint32_t)nxt;
    s.y = (uint32_t)(nxt >> 32);
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return __funnelshift_r(xs, xs, rot);
}

template <int RNG>
__device__ __forceinline__ uint32_t rng_next(uint4& s) {
    if constexpr (RNG == 1) return pcg32_next(s);
    else return xs128_next(s);
}

// random_move.comp:738-746: f = float(u) * 2^-32 (exact scale), then
// uint(ceil(float(min) + f * float(max - min + 1))) - 1 with separate roundings.
__device__ __forceinline__ uint32_t ranged(uint32_t u, uint32_t lo, uint32_t hi) {
    float f = __fmul_rn(__uint2float_rn(u), 2.3283064365386962890625e-10f);
    float v = __fadd_rn(__uint2float_rn(lo), __fmul_rn(f, __uint2float_rn(hi - lo + 1u)));
    return (uint32_t)ceilf(v) - 1u;
}

// splitmix64-based counter draws (same as the host initializer)
__host__ __device__ __forceinline__ uint64_t d_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t d_draw(uint64_t seed, uint64_t stream, uint64_t i) {
    return d_splitmix64(d_splitmix64(seed + 0x632BE59BD9B4E019ULL * stream) + i);
}
__device__ __forceinline__ float unit24(uint64_t d) {
    return __fmul_rn(__uint2float_rn((uint32_t)(d >> 40)), 5.9604644775390625e-8f);
}

// ---- move step --------------------------------------------------------------
// One tick of the move dispatch for one entity (random_move.comp:869-874):
// update_direction (:830-839) + move (:841-852) + new_target (:778-828).
// SPEED (:750) is generalised to step = (speed * factor[road]) * dt.
// The RNG state is loaded from rng_src only when a draw is needed.
template <int RNG>
__device__ __forceinline__ void step_entity(const DeviceMap& m, float dt, float speed, float2& p,
                                            uint32_t& h, uint4& r, bool& r_loaded, bool& r_dirty,
                                            const uint4* rng_src, uint32_t* err) {
    uint32_t road = h & kHeadRoad;
    bool to_end = (h & kHeadToEnd) != 0;
    if (road >= m.num_roads) {  // unreachable for validated inputs; never fault
        atomicOr(err, kErrOob);
        return;
    }
    float4 rp = __ldg(&m.road_pos[road]);
    float tx = to_end ? rp.z : rp.x;
    float ty = to_end ? rp.w : rp.y;
    float f = m.factor ? __ldg(&m.factor[road]) : 1.0f;
    float step = __fmul_rn(__fmul_rn(speed, f), dt);
    float dx = __fsub_rn(tx, p.x);
    float dy = __fsub_rn(ty, p.y);
    float len = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    if (len > step) {
        p.x = __fadd_rn(p.x, __fmul_rn(__fdiv_rn(dx, len), step));
        p.y = __fadd_rn(p.y, __fmul_rn(__fdiv_rn(dy, len), step));
        return;
    }
    // snap to the target; the leftover distance is discarded (:847-851)
    p.x = tx;
    p.y = ty;
    uint4 rc = __ldg(&m.road_conn[road]);
    uint32_t cidx = to_end ? rc.z : rc.x;
    uint32_t ccnt = to_end ? rc.w : rc.y;
    if (ccnt <= 1) {  // U-turn on the same road (:786-801)
        h = to_end ? road : (road | kHeadToEnd);
        return;
    }
    uint32_t off = 1;  // connectedCount == 2 -> connections[idx + 1] (:805-806)
    if (ccnt != 2) {   // ranged draw in [1, count], can return 0 or count (:808-811)
        if (!r_loaded) {
            r = *rng_src;
            r_loaded = true;
        }
        off = ranged(rng_next<RNG>(r), 1u, ccnt);
        r_dirty = true;
    }
    uint32_t ci = cidx + off;
    if (ci > m.num_conn) {  // unreachable after map validation
        atomicOr(err, kErrOob);
        ci = m.num_conn;
    }
    uint32_t nr = __ldg(&m.conn[ci]);
    if (nr >= m.num_roads) {
        atomicOr(err, kErrOob);
        return;
    }
    float4 np = __ldg(&m.road_pos[nr]);
    h = (np.x == tx && np.y == ty) ? (nr | kHeadToEnd) : nr;  // (:814-820)
}

// ---- spatial keys -------------------------------------------------------------
__host__ __device__ __forceinline__ constexpr uint32_t part1by1(uint32_t x) {
    x &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}
__host__ __device__ __forceinline__ uint32_t morton2(uint32_t x, uint32_t y) {
    return part1by1(x) | (part1by1(y) << 1);
}
// Tile coordinates are below 2^11: their bit spreads come from a constant table.
// For the query only, whose lanes hold consecutive sorted entries and so mostly
// share tiles (the constant cache broadcasts); divergent indices serialise.
struct MortonTable {
    uint32_t v[2048];
};
constexpr MortonTable make_morton_table() {
    MortonTable t{};
    for (uint32_t i = 0; i < 2048; i++) t.v[i] = part1by1(i);
    return t;
}
static __constant__ MortonTable c_morton = make_morton_table();
__device__ __forceinline__ uint32_t morton2_tile(uint32_t x, uint32_t y) {
    return c_morton.v[x & 2047u] | (c_morton.v[y & 2047u] << 1);
}
// Morton code of the tile one step up in x (or y): add 1 to the interleaved x (y)
// bits, carrying through the other axis' bits.
__host__ __device__ __forceinline__ uint32_t morton_inc_x(uint32_t m) {
    return (((m | 0xAAAAAAAAu) + 1u) & 0x55555555u) | (m & 0xAAAAAAAAu);
}
__host__ __device__ __forceinline__ uint32_t morton_inc_y(uint32_t m) {
    return (((m | 0x55555555u) + 2u) & 0xAAAAAAAAu) | (m & 0x55555555u);
}
// Tile coordinate: floor(v / cell) clamped to [0, n-1]; NaN maps to 0.  Monotone
// in v, so a query box [v - reach, v + reach] maps to a tile interval that holds
// every tile an in-range entity can occupy.
__device__ __forceinline__ uint32_t tile_coord(float v, float inv, uint32_t n) {
    float t = floorf(__fmul_rn(v, inv));
    if (!(t >= 0.f)) return 0u;
    if (t >= (float)n) return n - 1u;
    return (uint32_t)t;
}
// Band of y inside tile row ty: floor((y / cell - ty) * 2^ybits) clamped to the
// band range.  Monotone in y for a fixed ty, so the bands of an in-range entity
// lie between the bands of the query box's lower and upper y.
__device__ __forceinline__ uint32_t y_band(const TileGrid& g, float y, uint32_t ty) {
    const float f = floorf(__fmul_rn(__fsub_rn(__fmul_rn(y, g.inv_cell), (float)ty), g.ybands));
    if (!(f >= 0.f)) return 0u;
    if (f >= g.ybands) return (1u << g.ybits) - 1u;
    return (uint32_t)f;
}
// Sort key of a position.  mtab: the 2048 bit spreads part1by1(i), in shared
// memory (kernels over entities in any order: lanes with different tiles cost a
// bank conflict at worst, where the constant cache would serialise them).
__device__ __forceinline__ uint32_t tile_key(const TileGrid& g, float2 p, const uint32_t* mtab) {
    const uint32_t ty = tile_coord(p.y, g.inv_cell, g.tiles_y);
    const uint32_t tx = tile_coord(p.x, g.inv_cell, g.tiles_x);
    const uint32_t t = mtab[tx & 2047u] | (mtab[ty & 2047u] << 1);
    return g.ybits ? ((t << g.ybits) | y_band(g, p.y, ty)) : t;
}

// random_move.comp:551-562 quad_tree_in_range(v1 = other, v2 = self, R):
// |dx| <= R && |dy| <= R && length(v1 - v2) < R
__device__ __forceinline__ bool in_range(float2 other, float2 self, float r) {
    float dx = fabsf(__fsub_rn(self.x, other.x));
    if (dx > r) return false;
    float dy = fabsf(__fsub_rn(self.y, other.y));
    if (dy > r) return false;
    float ex = __fsub_rn(other.x, self.x);
    float ey = __fsub_rn(other.y, self.y);
    return __fsqrt_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey))) < r;
}

// The same predicate without the square root and without branches.  The
// correctly rounded square root is monotone, so sqrt_rn(d2) < r holds exactly
// when d2 < d2_limit, the smallest float whose rounded root reaches r.
__device__ __forceinline__ bool in_range_fast(float2 other, float2 self, float r, float d2_limit) {
    const float ex = __fsub_rn(other.x, self.x);
    const float ey = __fsub_rn(other.y, self.y);
    const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
    // |fl(a - b)| == |fl(b - a)|: the first two tests are those of in_range
    return (fabsf(ex) <= r) & (fabsf(ey) <= r) & (d2 < d2_limit);
}

// Smallest float t >= 0 whose correctly rounded square root is >= r (host side).
inline float sqrt_limit(float r) {
    if (!(r > 0.f)) return 0.f;
    float t = r * r;  // near the boundary; walk to the exact threshold
    while (t > 0.f && std::sqrt(std::nextafter(t, 0.f)) >= r) t = std::nextafter(t, 0.f);
    while (std::sqrt(t) < r) t = std::nextafter(t, INFINITY);
    return t;
}

}  // namespace msim
