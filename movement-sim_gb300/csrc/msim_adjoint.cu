// Differentiable density calibration: forward run with a time-averaged bilinear
// density splat, MSE loss against a target density, and the hand-written adjoint
// of the kinematic step with respect to per-entity speeds and per-road speed
// factors.
//
// Forward (k_adj_forward, one thread per entity, all ticks in registers): the
// move step of the plain path with step length speed*factor[road]*dt; every K
// ticks the state is checkpointed; each position is splatted with cell-centred
// bilinear weights into a gw x gh grid over the world.  Weights are accumulated
// per entity in registers as fixed point (units of 2^-31) while the entity stays in
// the same 2 x 2 cell block and flushed with 64-bit integer atomics when it leaves:
// integer addition is associative, so the density is bit-identical from run to
// run whatever the order of the flushes.
//
// Discrete events (the tick at which an entity reaches its road end and the road
// it picks) are held fixed: the gradient is that of the piecewise-smooth model
// with the forward's event schedule.  Every natural forward stores the schedule
// (one bit per entity and tick); a forward can replay it, so that finite
// differences can be taken on the same model, and the backward always does.
//
// Backward, per segment of K ticks from the last to the first
// (k_adj_backward): recompute the segment from its checkpoint with the recorded
// events, store positions and headings, then sweep backwards:
//   a_t += (1/T) d splat(p_t)/dp . lambda,     lambda = dL/dD = 2/G (D - D*)
//   snap tick:     a_{t-1} = 0 (p_t = road end does not depend on p, speed, factor)
//   otherwise:     n = (target - p_{t-1})/L, l = s*f*dt, g = n . a_t
//                  dL/ds += g*f*dt,  dL/df_road += g*s*dt,
//                  a_{t-1} = a_t - (l/L)(a_t - n g)
// Speed gradients are owned by their entity (no reduction).  Road-factor
// contributions are flushed as (road, value) records, one per road visit per
// segment, then sorted by road with the stable onesweep radix sort and summed per
// road in record order: a deterministic segmented reduction, no float atomics.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "msim_internal.h"
#include "msim_kernels.cuh"

namespace msim {
namespace {

constexpr uint32_t kRecPerSeg = 8;  // road-visit records per entity and segment
constexpr uint32_t kSnapBit = 1u << 30;

struct AdjArgs {
    DeviceMap map;
    uint32_t n, ticks, K, sched_words;
    float dt, inv_cw, inv_ch;
    uint32_t gw, gh, fbits;
    const float2* pos0;
    const uint32_t* head0;
    const uint4* rng0;
    const float* speed;
    float2* ck_pos;
    uint32_t* ck_head;
    uint4* ck_rng;
    unsigned long long* dacc;
    uint32_t* sched;  // one bit per entity and tick
    uint32_t mode;    // 0 / 1 natural (the schedule is stored), 2 replay the stored schedule
    uint32_t* err;
};

// One tick; returns whether the entity snapped to its road end.  force < 0:
// natural decision (len <= step); 0 / 1: the recorded decision.
template <int RNG>
__device__ __forceinline__ bool adj_step(const DeviceMap& m, float dt, float speed, float2& p, uint32_t& h, uint4& r,
                                         int force, uint32_t* err) {
    const uint32_t road = h & kHeadRoad;
    if (road >= m.num_roads) {
        atomicOr(err, kErrOob);
        return false;
    }
    const bool to_end = (h & kHeadToEnd) != 0;
    const float4 rp = __ldg(&m.road_pos[road]);
    const float tx = to_end ? rp.z : rp.x, ty = to_end ? rp.w : rp.y;
    const float f = m.factor ? __ldg(&m.factor[road]) : 1.0f;
    const float step = __fmul_rn(__fmul_rn(speed, f), dt);
    const float dx = __fsub_rn(tx, p.x), dy = __fsub_rn(ty, p.y);
    const float len = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    const bool snap = force < 0 ? !(len > step) : force != 0;
    if (!snap) {
        if (len > 0.f) {
            p.x = __fadd_rn(p.x, __fmul_rn(__fdiv_rn(dx, len), step));
            p.y = __fadd_rn(p.y, __fmul_rn(__fdiv_rn(dy, len), step));
        }
        return false;
    }
    p.x = tx;
    p.y = ty;
    const uint4 rc = __ldg(&m.road_conn[road]);
    const uint32_t cidx = to_end ? rc.z : rc.x, ccnt = to_end ? rc.w : rc.y;
    if (ccnt <= 1) {
        h = to_end ? road : (road | kHeadToEnd);
        return true;
    }
    uint32_t off = 1;
    if (ccnt != 2) off = ranged(rng_next<RNG>(r), 1u, ccnt);
    uint32_t ci = cidx + off;
    if (ci > m.num_conn) {
        atomicOr(err, kErrOob);
        ci = m.num_conn;
    }
    const uint32_t nr = __ldg(&m.conn[ci]);
    if (nr >= m.num_roads) {
        atomicOr(err, kErrOob);
        return true;
    }
    const float4 np = __ldg(&m.road_pos[nr]);
    h = (np.x == tx && np.y == ty) ? (nr | kHeadToEnd) : nr;
    return true;
}

// Cell coordinates of a position: u = x * (gw / W) - 1/2 in binary32 (cell-centred),
// then U = floor(u * 2^fbits) as an integer (exact: a binary32 u below 2^(30-fbits)
// has no fractional bits beyond fbits once truncated there).  The cell is
// U >> fbits and the fraction fx = (U mod 2^fbits) / 2^fbits; fbits is the largest
// value (at most 22) that keeps U in 31 bits for the grid.
struct Splat {
    int i0, j0;
    uint32_t fx, fy;  // fractions in units of 2^-fbits
};
__device__ __forceinline__ int fixed_coord(float u, uint32_t fbits) {
    const float lim = __int_as_float((127 + 30 - (int)fbits) << 23);  // 2^(30 - fbits)
    u = fminf(fmaxf(u, -lim), lim);                                  // off-grid positions stay off-grid
    return __float2int_rd(__fmul_rn(u, __int_as_float((127 + (int)fbits) << 23)));
}
__device__ __forceinline__ Splat splat_of(float x, float y, float inv_cw, float inv_ch, uint32_t fbits) {
    const int U = fixed_coord(__fsub_rn(__fmul_rn(x, inv_cw), 0.5f), fbits);
    const int V = fixed_coord(__fsub_rn(__fmul_rn(y, inv_ch), 0.5f), fbits);
    const uint32_t mask = (1u << fbits) - 1u;
    Splat s;
    s.i0 = U >> fbits;  // arithmetic shift: floor
    s.j0 = V >> fbits;
    s.fx = (uint32_t)U & mask;
    s.fy = (uint32_t)V & mask;
    return s;
}
// Per-entity sums over the ticks spent in one 2 x 2 cell block: the tick count and
// the sums of fx, fy and fx*fy give the four bilinear corner weights exactly.
struct BlockSums {
    uint32_t n;
    unsigned long long sx, sy, sxy;
};
__device__ __forceinline__ void flush_block(unsigned long long* dacc, uint32_t gw, uint32_t gh, int i0, int j0,
                                            const BlockSums& b, uint32_t fbits) {
    const unsigned long long F = 1ull << fbits;
    // corner weights in units of 2^-2fbits, then in the accumulator's 2^-31
    const unsigned long long w[4] = {(unsigned long long)b.n * F * F - F * (b.sx + b.sy) + b.sxy, F * b.sx - b.sxy,
                                     F * b.sy - b.sxy, b.sxy};
    const uint32_t sh = 2u * fbits - 31u;
    const int ci[4] = {i0, i0 + 1, i0, i0 + 1}, cj[4] = {j0, j0, j0 + 1, j0 + 1};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const unsigned long long v = w[k] >> sh;
        if (v && ci[k] >= 0 && cj[k] >= 0 && ci[k] < (int)gw && cj[k] < (int)gh)
            atomicAdd(&dacc[(size_t)cj[k] * gw + ci[k]], v);
    }
}

template <int RNG>
__global__ __launch_bounds__(256) void k_adj_forward(AdjArgs a) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.n) return;
    float2 p = a.pos0[e];
    uint32_t h = a.head0[e];
    uint4 r = a.rng0[e];
    const float s = a.speed[e];
    int bi = INT32_MIN, bj = INT32_MIN;
    BlockSums acc{0u, 0ull, 0ull, 0ull};
    uint32_t bits = 0;
    uint32_t until_ck = 0;  // ticks until the next checkpoint
    size_t ck = e;
    for (uint32_t t = 1; t <= a.ticks; t++) {
        if (until_ck == 0) {
            a.ck_pos[ck] = p;
            a.ck_head[ck] = h;
            a.ck_rng[ck] = r;
            ck += a.n;
            until_ck = a.K;
        }
        until_ck--;
        const uint32_t w = (t - 1) >> 5, b = (t - 1) & 31u;
        int force = -1;
        if (a.mode == 2) force = (a.sched[(size_t)e * a.sched_words + w] >> b) & 1u;
        const bool snapped = RNG == 1 ? adj_step<1>(a.map, a.dt, s, p, h, r, force, a.err)
                                      : adj_step<0>(a.map, a.dt, s, p, h, r, force, a.err);
        if (a.mode != 2) {  // the schedule of the last forward, replayed by the backward
            if (snapped) bits |= 1u << b;
            if (b == 31 || t == a.ticks) {
                a.sched[(size_t)e * a.sched_words + w] = bits;
                bits = 0;
            }
        }
        const Splat sp = splat_of(p.x, p.y, a.inv_cw, a.inv_ch, a.fbits);
        if (sp.i0 != bi || sp.j0 != bj) {
            if (bi != INT32_MIN) flush_block(a.dacc, a.gw, a.gh, bi, bj, acc, a.fbits);
            bi = sp.i0;
            bj = sp.j0;
            acc = BlockSums{0u, 0ull, 0ull, 0ull};
        }
        acc.n++;
        acc.sx += sp.fx;
        acc.sy += sp.fy;
        acc.sxy += (unsigned long long)sp.fx * sp.fy;
    }
    if (bi != INT32_MIN) flush_block(a.dacc, a.gw, a.gh, bi, bj, acc, a.fbits);
}

// density, lambda = 2/G (D - D*), per-block partial sums of (D - D*)^2
__global__ __launch_bounds__(256) void k_adj_loss(const unsigned long long* __restrict__ dacc,
                                                  const float* __restrict__ target, uint32_t G, uint32_t ticks,
                                                  float* density, float* lambda, double* partial) {
    __shared__ double s_sum[256];
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    double d2 = 0.0;
    if (g < G) {
        const double D = (double)dacc[g] * 0x1p-31 / (double)ticks;
        const double diff = D - (double)target[g];
        density[g] = (float)D;
        lambda[g] = (float)(2.0 / (double)G * diff);
        d2 = diff * diff;
    }
    s_sum[threadIdx.x] = d2;
    __syncthreads();
    for (uint32_t o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s_sum[threadIdx.x] += s_sum[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s_sum[0];
}

__global__ void k_adj_loss_final(const double* partial, uint32_t blocks, uint32_t G, double* loss) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double s = 0.0;
    for (uint32_t b = 0; b < blocks; b++) s += partial[b];
    *loss = s / (double)G;
}

struct AdjBack {
    AdjArgs f;
    uint32_t seg;
    const float* lambda;
    float2* hist_pos;     // [K][n]
    uint32_t* hist_head;  // [K][n], heading before the tick | snap bit
    float2* carry;        // adjoint of the position at the segment's end
    double* gspeed;
    uint32_t* rec_road;   // [segments][n][kRecPerSeg], unused = num_roads
    double* rec_val;
    uint32_t num_roads;
};

__device__ __forceinline__ float lam_at(const float* lambda, uint32_t gw, uint32_t gh, int i, int j) {
    return (i < 0 || j < 0 || i >= (int)gw || j >= (int)gh) ? 0.f : __ldg(&lambda[(size_t)j * gw + i]);
}

// The recorded step for the backward's recompute: the event decision comes from the
// schedule, the road choice from the checkpointed RNG (both exact); the position
// update uses the hardware reciprocal square root, since the adjoint needs the
// positions only to about 1e-6 relative (snaps put them back on exact road ends).
template <int RNG>
__device__ __forceinline__ void adj_replay_step(const DeviceMap& m, float dt, float speed, float2& p, uint32_t& h,
                                                uint4& r, bool snap, uint32_t* err) {
    const uint32_t road = h & kHeadRoad;
    if (road >= m.num_roads) {
        atomicOr(err, kErrOob);
        return;
    }
    const bool to_end = (h & kHeadToEnd) != 0;
    const float4 rp = __ldg(&m.road_pos[road]);
    const float tx = to_end ? rp.z : rp.x, ty = to_end ? rp.w : rp.y;
    if (!snap) {
        const float f = m.factor ? __ldg(&m.factor[road]) : 1.0f;
        const float step = speed * f * dt;
        const float dx = tx - p.x, dy = ty - p.y;
        const float d2 = dx * dx + dy * dy;
        if (d2 > 0.f) {
            const float k = rsqrtf(d2) * step;
            p.x += dx * k;
            p.y += dy * k;
        }
        return;
    }
    p.x = tx;
    p.y = ty;
    const uint4 rc = __ldg(&m.road_conn[road]);
    const uint32_t cidx = to_end ? rc.z : rc.x, ccnt = to_end ? rc.w : rc.y;
    if (ccnt <= 1) {
        h = to_end ? road : (road | kHeadToEnd);
        return;
    }
    uint32_t off = 1;
    if (ccnt != 2) off = ranged(rng_next<RNG>(r), 1u, ccnt);
    uint32_t ci = cidx + off;
    if (ci > m.num_conn) {
        atomicOr(err, kErrOob);
        ci = m.num_conn;
    }
    const uint32_t nr = __ldg(&m.conn[ci]);
    if (nr >= m.num_roads) {
        atomicOr(err, kErrOob);
        return;
    }
    const float4 np = __ldg(&m.road_pos[nr]);
    h = (np.x == tx && np.y == ty) ? (nr | kHeadToEnd) : nr;
}

// lambda at the four corners of p's cell block, and the fractions
struct SplatLam {
    float l00, l10, l01, l11, fx, fy;
};
__device__ __forceinline__ SplatLam splat_lam(const AdjBack& b, float2 p) {
    const Splat sp = splat_of(p.x, p.y, b.f.inv_cw, b.f.inv_ch, b.f.fbits);
    const float scale = __int_as_float((127 - (int)b.f.fbits) << 23);  // 2^-fbits
    SplatLam o;
    o.l00 = lam_at(b.lambda, b.f.gw, b.f.gh, sp.i0, sp.j0);
    o.l10 = lam_at(b.lambda, b.f.gw, b.f.gh, sp.i0 + 1, sp.j0);
    o.l01 = lam_at(b.lambda, b.f.gw, b.f.gh, sp.i0, sp.j0 + 1);
    o.l11 = lam_at(b.lambda, b.f.gw, b.f.gh, sp.i0 + 1, sp.j0 + 1);
    o.fx = (float)sp.fx * scale;  // exact: fewer than 24 bits
    o.fy = (float)sp.fy * scale;
    return o;
}

template <int RNG>
__global__ __launch_bounds__(256) void k_adj_backward(AdjBack b) {
    const AdjArgs& a = b.f;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.n) return;
    const uint32_t t0 = b.seg * a.K + 1, t1 = min((b.seg + 1) * a.K, a.ticks);
    const size_t ck = (size_t)b.seg * a.n + e;
    const float2 pk = a.ck_pos[ck];
    float2 p = pk;
    uint32_t h = a.ck_head[ck];
    uint4 r = a.ck_rng[ck];
    const float s = a.speed[e];
    const uint32_t* sched = a.sched + (size_t)e * a.sched_words;
    uint32_t word = 0;
    for (uint32_t t = t0; t <= t1; t++) {  // recompute the segment with the recorded events
        const uint32_t bit = (t - 1) & 31u;
        if (t == t0 || bit == 0) word = sched[(t - 1) >> 5];
        const bool snap = (word >> bit) & 1u;
        const uint32_t hb = h;
        adj_replay_step<RNG>(a.map, a.dt, s, p, h, r, snap, a.err);
        const size_t hi = (size_t)(t - t0) * a.n + e;
        b.hist_pos[hi] = p;
        b.hist_head[hi] = hb | (snap ? kSnapBit : 0u);
    }
    // reverse sweep; positions, headings and lambda are fetched one tick ahead
    float2 adj = b.carry[e];
    float gs = 0.f, cur_sum = 0.f;
    uint32_t cur_road = b.num_roads, nrec = 0;
    const size_t rec0 = ((size_t)b.seg * a.n + e) * kRecPerSeg;
    const float sx = a.inv_cw, sy = a.inv_ch, invT = 1.0f / (float)a.ticks;
    const size_t n = a.n;
    float2 pt = b.hist_pos[(size_t)(t1 - t0) * n + e];
    uint32_t hw = b.hist_head[(size_t)(t1 - t0) * n + e];
    float2 pp = t1 > t0 ? b.hist_pos[(size_t)(t1 - 1 - t0) * n + e] : pk;
    SplatLam sl = splat_lam(b, pt);
    for (uint32_t t = t1;; t--) {
        uint32_t hw_n = 0;
        float2 pp_n = pk;
        if (t > t0) {
            hw_n = b.hist_head[(size_t)(t - 1 - t0) * n + e];
            if (t - 1 > t0) pp_n = b.hist_pos[(size_t)(t - 2 - t0) * n + e];
        }
        const SplatLam sl_n = splat_lam(b, pp);  // lambda for the next (earlier) tick
        {  // + (1/T) d splat(p_t)/dp . lambda
            const float gx = ((1.f - sl.fy) * (sl.l10 - sl.l00) + sl.fy * (sl.l11 - sl.l01)) * sx;
            const float gy = ((1.f - sl.fx) * (sl.l01 - sl.l00) + sl.fx * (sl.l11 - sl.l10)) * sy;
            adj.x += gx * invT;
            adj.y += gy * invT;
        }
        if (hw & kSnapBit) {
            adj = make_float2(0.f, 0.f);
        } else {
            const uint32_t h0 = hw & ~kSnapBit;
            const uint32_t road = h0 & kHeadRoad;
            const float4 rp = __ldg(&a.map.road_pos[road]);
            const float tx = (h0 & kHeadToEnd) ? rp.z : rp.x, ty = (h0 & kHeadToEnd) ? rp.w : rp.y;
            const float dx = tx - pp.x, dy = ty - pp.y;
            const float d2 = dx * dx + dy * dy;
            if (d2 > 0.f) {
                const float invL = rsqrtf(d2);
                const float f = a.map.factor ? __ldg(&a.map.factor[road]) : 1.0f;
                const float nx = dx * invL, ny = dy * invL;
                const float g = nx * adj.x + ny * adj.y;
                gs += g * f * a.dt;
                if (road != cur_road) {
                    if (cur_road != b.num_roads) {
                        if (nrec < kRecPerSeg) {
                            b.rec_road[rec0 + nrec] = cur_road;
                            b.rec_val[rec0 + nrec] = (double)cur_sum;
                            nrec++;
                        } else {
                            atomicOr(a.err, kErrOob);
                        }
                    }
                    cur_road = road;
                    cur_sum = 0.f;
                }
                cur_sum += g * s * a.dt;
                const float k = s * f * a.dt * invL;
                adj.x -= k * (adj.x - nx * g);
                adj.y -= k * (adj.y - ny * g);
            }
        }
        if (t == t0) break;
        pt = pp;
        pp = pp_n;
        hw = hw_n;
        sl = sl_n;
    }
    if (cur_road != b.num_roads) {
        if (nrec < kRecPerSeg) {
            b.rec_road[rec0 + nrec] = cur_road;
            b.rec_val[rec0 + nrec] = (double)cur_sum;
            nrec++;
        } else {
            atomicOr(a.err, kErrOob);
        }
    }
    for (uint32_t j = nrec; j < kRecPerSeg; j++) {
        b.rec_road[rec0 + j] = b.num_roads;
        b.rec_val[rec0 + j] = 0.0;
    }
    b.carry[e] = adj;
    b.gspeed[e] += (double)gs;
}

// sum of every road's records in sorted (stable) order
__global__ void k_adj_road_sum(const uint32_t* __restrict__ kstart, const uint32_t* __restrict__ sorted_rec,
                               const double* __restrict__ rec_val, uint32_t num_roads, uint32_t total,
                               double* gfactor, float* out) {
    const uint32_t rd = blockIdx.x * blockDim.x + threadIdx.x;
    if (rd >= num_roads) return;
    const uint32_t lo = kstart[rd], hi = min(kstart[rd + 1], total);
    double s = 0.0;
    for (uint32_t q = lo; q < hi; q++) s += rec_val[sorted_rec[q]];
    gfactor[rd] = s;
    if (out) out[rd] = (float)s;
}

// Entities are kept in spatial order inside the context (perm[i] = entity id of
// internal index i); these move per-entity arrays across that boundary.
__global__ void k_adj_speed_out(const double* gspeed, const uint32_t* perm, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = (float)gspeed[i];
}
__global__ void k_adj_gather(const float* __restrict__ in, const uint32_t* __restrict__ perm, uint32_t n,
                             float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[perm[i]];
}

// Digit histograms of the record keys for the radix sort (keys < 2^(8*passes)).
__global__ void k_adj_hist(const uint32_t* __restrict__ keys, size_t count, uint32_t passes, uint32_t* hist) {
    __shared__ uint32_t s_hist[kMaxPasses * kRadix];
    for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        for (uint32_t ps = 0; ps < passes; ps++) atomicAdd(&s_hist[ps * kRadix + ((k >> (8 * ps)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], s_hist[i]);
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MSIM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define ACK(expr, what)                                    \
    do {                                                   \
        cudaError_t e_ = (expr);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

}  // namespace
}  // namespace msim

using namespace msim;

struct msim_adj {
    int device = 0;
    cudaStream_t stream = nullptr;
    msim_adj_params p{};
    uint32_t n = 0, R = 0, C = 0, S = 0, sched_words = 0, passes = 1;
    float world_w = 0, world_h = 0;
    std::vector<void*> allocs;
    float4* road_pos = nullptr;
    uint4* road_conn = nullptr;
    uint32_t* conn = nullptr;
    float* speed = nullptr;
    float* factor = nullptr;
    float* target = nullptr;
    float2* pos0 = nullptr;
    uint32_t* head0 = nullptr;
    uint4* rng0 = nullptr;
    float2* ck_pos = nullptr;
    uint32_t* ck_head = nullptr;
    uint4* ck_rng = nullptr;
    unsigned long long* dacc = nullptr;
    float* density = nullptr;
    float* lambda = nullptr;
    double* partial = nullptr;
    double* loss = nullptr;
    uint32_t* sched = nullptr;
    float2* hist_pos = nullptr;
    uint32_t* hist_head = nullptr;
    float2* carry = nullptr;
    double* gspeed = nullptr;
    double* gfactor = nullptr;
    uint32_t* rec_road = nullptr;
    double* rec_val = nullptr;
    uint32_t* sk[2] = {nullptr, nullptr};
    uint32_t* sv[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;
    uint32_t* lookback = nullptr;
    uint32_t* tickets = nullptr;
    uint32_t* kstart = nullptr;
    uint32_t* err = nullptr;
    uint32_t* perm = nullptr;        // device: entity id of each internal index
    std::vector<uint32_t> hperm;     // host copy
    size_t rec_count = 0;
    uint32_t rec_tiles = 0;
    bool have_forward = false;
    bool have_backward = false;
    bool have_sched = false;
    uint32_t last_mode = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaEvent_t ph[6] = {};  // forward: kernel start/end, loss end; backward: start, sweeps end, end
};

namespace {

template <typename T>
int aalloc(msim_adj* a, T** ptr, size_t count) {
    void* raw = nullptr;
    if (!device_malloc(&raw, std::max<size_t>(count, 1) * sizeof(T)))
        return fail(MSIM_ERR_NOMEM, "device allocation failed in the adjoint context");
    a->allocs.push_back(raw);
    *ptr = static_cast<T*>(raw);
    return MSIM_OK;
}

void free_adj(msim_adj* a) {
    for (void* p : a->allocs) cudaFree(p);
    a->allocs.clear();
    if (a->t0) cudaEventDestroy(a->t0);
    if (a->t1) cudaEventDestroy(a->t1);
    for (cudaEvent_t& ev : a->ph)
        if (ev) cudaEventDestroy(ev);
    if (a->stream) cudaStreamDestroy(a->stream);
}

// Fraction bits of the splat's fixed-point cell coordinates: the largest value
// (at most 22, at least 16) with |u| * 2^fbits below 2^30 for u in (-1, max(gw, gh)).
uint32_t splat_fraction_bits(uint32_t gw, uint32_t gh) {
    const uint32_t g = std::max(gw, gh);
    uint32_t b = 0;
    while ((1ull << b) < (uint64_t)g + 1u) b++;
    const int fb = 30 - (int)b;
    return (uint32_t)std::max(16, std::min(22, fb));
}

AdjArgs fwd_args(msim_adj* a, uint32_t mode) {
    AdjArgs f{};
    f.map.road_pos = a->road_pos;
    f.map.road_conn = a->road_conn;
    f.map.conn = a->conn;
    f.map.factor = a->factor;
    f.map.num_roads = a->R;
    f.map.num_conn = a->C;
    f.n = a->n;
    f.ticks = a->p.ticks;
    f.K = a->p.checkpoint_interval;
    f.sched_words = a->sched_words;
    f.dt = a->p.dt;
    f.inv_cw = (float)((double)a->p.grid_w / (double)a->world_w);
    f.inv_ch = (float)((double)a->p.grid_h / (double)a->world_h);
    f.fbits = splat_fraction_bits(a->p.grid_w, a->p.grid_h);
    f.gw = a->p.grid_w;
    f.gh = a->p.grid_h;
    f.pos0 = a->pos0;
    f.head0 = a->head0;
    f.rng0 = a->rng0;
    f.speed = a->speed;
    f.ck_pos = a->ck_pos;
    f.ck_head = a->ck_head;
    f.ck_rng = a->ck_rng;
    f.dacc = a->dacc;
    f.sched = a->sched;
    f.mode = mode;
    f.err = a->err;
    return f;
}

int check_status(msim_adj* a) {
    ACK(cudaStreamSynchronize(a->stream), "cudaStreamSynchronize");
    uint32_t h = 0;
    ACK(cudaMemcpy(&h, a->err, sizeof(h), cudaMemcpyDeviceToHost), "read device status");
    if (h) {
        ACK(cudaMemset(a->err, 0, sizeof(uint32_t)), "clear device status");
        if (h & kErrTimeout) return fail(MSIM_ERR_TIMEOUT, "a bounded device wait gave up in the road-gradient sort");
        return fail(MSIM_ERR_OOB, "device-side index check failed in the adjoint (or more than 8 road visits per "
                                  "entity in one checkpoint segment)");
    }
    return MSIM_OK;
}

}  // namespace

namespace {
// host scatter of an internal-order array to entity-id order
template <typename T>
void to_entity_order(const std::vector<uint32_t>& perm, const T* in, T* out, size_t width = 1) {
    for (size_t i = 0; i < perm.size(); i++)
        for (size_t w = 0; w < width; w++) out[(size_t)perm[i] * width + w] = in[i * width + w];
}
}  // namespace

extern "C" {

int msim_adj_create(const msim_map* map, const msim_adj_params* params, msim_adj** out) {
    if (!out) return fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!map || !params) return fail(MSIM_ERR_INVALID, "NULL argument");
    int rc = validate_map(*map);
    if (rc != MSIM_OK) return rc;
    const msim_adj_params& p = *params;
    if (p.num_entities == 0 || p.num_entities >= (1u << 28)) return fail(MSIM_ERR_INVALID, "num_entities out of range");
    if (p.ticks == 0 || p.checkpoint_interval == 0) return fail(MSIM_ERR_INVALID, "ticks and checkpoint_interval must be > 0");
    if (p.grid_w == 0 || p.grid_h == 0 || (uint64_t)p.grid_w * p.grid_h > (1ull << 26) || p.grid_w > 16384u ||
        p.grid_h > 16384u)
        return fail(MSIM_ERR_INVALID, "density grid size out of range");
    if (p.rng_kind > 1 || p.placement > 1) return fail(MSIM_ERR_INVALID, "unknown rng_kind or placement");
    if (!(p.dt > 0.f) || !(p.speed_max >= p.speed_min)) return fail(MSIM_ERR_INVALID, "bad dt or speed range");
    if (map->num_roads >= (1u << 30)) return fail(MSIM_ERR_INVALID, "too many roads");
    msim_adj* a = new (std::nothrow) msim_adj();
    if (!a) return fail(MSIM_ERR_NOMEM, "out of host memory");
    auto bail = [&](int code) {
        free_adj(a);
        delete a;
        return code;
    };
    cudaGetDevice(&a->device);
    a->p = p;
    a->n = p.num_entities;
    a->R = map->num_roads;
    a->C = map->num_connections;
    a->world_w = map->width;
    a->world_h = map->height;
    a->S = (p.ticks + p.checkpoint_interval - 1) / p.checkpoint_interval;
    a->sched_words = (p.ticks + 31) / 32;
    uint32_t bits = 1;
    while ((1ull << bits) <= a->R) bits++;  // keys 0..R (R = unused record)
    a->passes = (bits + 7) / 8;
    if (a->passes > kMaxPasses) return bail(fail(MSIM_ERR_INVALID, "too many roads for the record sort"));
    a->rec_count = (size_t)a->S * a->n * kRecPerSeg;
    if (a->rec_count >= (1ull << 30)) return bail(fail(MSIM_ERR_INVALID, "ticks x entities too large for the record sort"));
    a->rec_tiles = (uint32_t)((a->rec_count + kSortTile - 1) / kSortTile);
    cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    cudaEventCreate(&a->t0);
    cudaEventCreate(&a->t1);
    for (cudaEvent_t& ev : a->ph) cudaEventCreate(&ev);
    const size_t n = a->n, G = (size_t)p.grid_w * p.grid_h, K = p.checkpoint_interval;
    if ((rc = aalloc(a, &a->road_pos, a->R)) || (rc = aalloc(a, &a->road_conn, a->R)) ||
        (rc = aalloc(a, &a->conn, (size_t)a->C + 1)) || (rc = aalloc(a, &a->speed, n)) ||
        (rc = aalloc(a, &a->factor, a->R)) || (rc = aalloc(a, &a->target, G)) || (rc = aalloc(a, &a->pos0, n)) ||
        (rc = aalloc(a, &a->head0, n)) || (rc = aalloc(a, &a->rng0, n)) || (rc = aalloc(a, &a->ck_pos, a->S * n)) ||
        (rc = aalloc(a, &a->ck_head, a->S * n)) || (rc = aalloc(a, &a->ck_rng, a->S * n)) ||
        (rc = aalloc(a, &a->dacc, G)) || (rc = aalloc(a, &a->density, G)) || (rc = aalloc(a, &a->lambda, G)) ||
        (rc = aalloc(a, &a->partial, (G + 255) / 256)) || (rc = aalloc(a, &a->loss, 1)) ||
        (rc = aalloc(a, &a->sched, n * a->sched_words)) || (rc = aalloc(a, &a->hist_pos, K * n)) ||
        (rc = aalloc(a, &a->hist_head, K * n)) || (rc = aalloc(a, &a->carry, n)) || (rc = aalloc(a, &a->gspeed, n)) ||
        (rc = aalloc(a, &a->gfactor, a->R)) || (rc = aalloc(a, &a->rec_road, a->rec_count)) ||
        (rc = aalloc(a, &a->rec_val, a->rec_count)) || (rc = aalloc(a, &a->sk[0], a->rec_count)) ||
        (rc = aalloc(a, &a->sk[1], a->rec_count)) || (rc = aalloc(a, &a->sv[0], a->rec_count)) ||
        (rc = aalloc(a, &a->sv[1], a->rec_count)) || (rc = aalloc(a, &a->hist, (size_t)kMaxPasses * kRadix)) ||
        (rc = aalloc(a, &a->lookback, (size_t)kMaxPasses * a->rec_tiles * kRadix)) ||
        (rc = aalloc(a, &a->tickets, (size_t)kMaxPasses)) || (rc = aalloc(a, &a->kstart, (size_t)a->R + 2)) ||
        (rc = aalloc(a, &a->err, 1)) || (rc = aalloc(a, &a->perm, n)))
        return bail(rc);
    std::vector<uint32_t> conn(a->C + 1);
    if (a->C) std::memcpy(conn.data(), map->connections, sizeof(uint32_t) * a->C);
    conn[a->C] = a->C ? map->connections[a->C - 1] : 0u;
    std::vector<float> ones(a->R, 1.0f);
    e = cudaMemcpy(a->road_pos, map->road_pos, sizeof(float4) * a->R, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(a->road_conn, map->road_conn, sizeof(uint4) * a->R, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(a->conn, conn.data(), sizeof(uint32_t) * (a->C + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(a->factor, ones.data(), sizeof(float) * a->R, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(a->err, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(a->target, 0, sizeof(float) * G);
    if (e != cudaSuccess) return bail(cuda_fail(e, "adjoint set-up"));
    // initial entity state: the deterministic initializer of msim_init_entities
    DeviceMap m{};
    m.road_pos = a->road_pos;
    m.road_conn = a->road_conn;
    m.conn = a->conn;
    m.num_roads = a->R;
    m.num_conn = a->C;
    EntityState st{};
    st.pos = a->pos0;
    st.head = a->head0;
    st.rng = a->rng0;
    st.speed = a->speed;
    st.slot_id = a->hist_head;  // scratch for the slot ids the initializer writes
    e = launch_init_entities(a->stream, m, st, a->n, p.rng_kind, p.seed, p.placement, p.speed_min, p.speed_max);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "adjoint entity init"));
    // spatial order: entities sorted (stably) by the Morton code of their initial
    // density cell, so a warp's cell gathers and flushes touch nearby cells
    {
        std::vector<float2> pos(n);
        std::vector<uint32_t> head(n), spd(n);
        std::vector<uint4> rng(n);
        e = cudaMemcpy(pos.data(), a->pos0, sizeof(float2) * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(head.data(), a->head0, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(rng.data(), a->rng0, sizeof(uint4) * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(spd.data(), a->speed, sizeof(float) * n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return bail(cuda_fail(e, "adjoint spatial order"));
        const double sx = (double)p.grid_w / (double)a->world_w, sy = (double)p.grid_h / (double)a->world_h;
        std::vector<uint32_t> key(n);
        for (size_t i = 0; i < n; i++) {
            const double cx = std::min(std::max((double)pos[i].x * sx, 0.0), (double)p.grid_w - 1.0);
            const double cy = std::min(std::max((double)pos[i].y * sy, 0.0), (double)p.grid_h - 1.0);
            key[i] = morton2((uint32_t)cx, (uint32_t)cy);
        }
        a->hperm.resize(n);
        for (size_t i = 0; i < n; i++) a->hperm[i] = (uint32_t)i;
        std::stable_sort(a->hperm.begin(), a->hperm.end(), [&](uint32_t x, uint32_t y) { return key[x] < key[y]; });
        std::vector<float2> pos2(n);
        std::vector<uint32_t> head2(n), spd2(n);
        std::vector<uint4> rng2(n);
        for (size_t i = 0; i < n; i++) {
            const uint32_t id = a->hperm[i];
            pos2[i] = pos[id];
            head2[i] = head[id];
            rng2[i] = rng[id];
            spd2[i] = spd[id];
        }
        e = cudaMemcpy(a->pos0, pos2.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(a->head0, head2.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(a->rng0, rng2.data(), sizeof(uint4) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(a->speed, spd2.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(a->perm, a->hperm.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "adjoint spatial order"));
    }
    *out = a;
    return MSIM_OK;
}


int msim_adj_destroy(msim_adj* a) {
    if (!a) return MSIM_OK;
    cudaSetDevice(a->device);
    cudaStreamSynchronize(a->stream);
    free_adj(a);
    delete a;
    return MSIM_OK;
}

int msim_adj_get_initial_state(msim_adj* a, float* pos, uint32_t* heading, uint32_t* rng, float* speed) {
    if (!a) return fail(MSIM_ERR_INVALID, "NULL argument");
    cudaSetDevice(a->device);
    ACK(cudaStreamSynchronize(a->stream), "sync");
    const size_t n = a->n;
    std::vector<uint32_t> tmp(4 * n);
    if (pos) {
        ACK(cudaMemcpy(tmp.data(), a->pos0, sizeof(float2) * n, cudaMemcpyDeviceToHost), "download");
        to_entity_order(a->hperm, reinterpret_cast<const float*>(tmp.data()), pos, 2);
    }
    if (heading) {
        ACK(cudaMemcpy(tmp.data(), a->head0, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost), "download");
        to_entity_order(a->hperm, tmp.data(), heading);
    }
    if (rng) {
        ACK(cudaMemcpy(tmp.data(), a->rng0, sizeof(uint4) * n, cudaMemcpyDeviceToHost), "download");
        to_entity_order(a->hperm, tmp.data(), rng, 4);
    }
    // the current speeds: the initializer's until a forward passes others
    if (speed) {
        ACK(cudaMemcpy(tmp.data(), a->speed, sizeof(float) * n, cudaMemcpyDeviceToHost), "download");
        to_entity_order(a->hperm, reinterpret_cast<const float*>(tmp.data()), speed);
    }
    return MSIM_OK;
}

int msim_adj_forward(msim_adj* a, const float* d_speed, const float* d_factor, const float* d_target,
                     float* d_density, uint32_t mode, double* loss) {
    msim::NvtxRange range("msim_adj_forward");
    if (!a) return fail(MSIM_ERR_INVALID, "NULL argument");
    if (mode > 2) return fail(MSIM_ERR_INVALID, "mode must be 0 (natural), 1 (record events) or 2 (replay events)");
    if (mode == 2 && !a->have_sched) return fail(MSIM_ERR_INVALID, "no recorded event schedule to replay");
    cudaSetDevice(a->device);
    const size_t n = a->n, G = (size_t)a->p.grid_w * a->p.grid_h;
    if (d_speed) {
        k_adj_gather<<<(unsigned)((n + 255) / 256), 256, 0, a->stream>>>(d_speed, a->perm, a->n, a->speed);
        ACK(cudaGetLastError(), "speed");
    }
    if (d_factor)
        ACK(cudaMemcpyAsync(a->factor, d_factor, sizeof(float) * a->R, cudaMemcpyDeviceToDevice, a->stream), "factor");
    if (d_target)
        ACK(cudaMemcpyAsync(a->target, d_target, sizeof(float) * G, cudaMemcpyDeviceToDevice, a->stream), "target");
    ACK(cudaMemsetAsync(a->dacc, 0, sizeof(unsigned long long) * G, a->stream), "memset density");
    AdjArgs f = fwd_args(a, mode);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaEventRecord(a->ph[0], a->stream);
    if (a->p.rng_kind == 1) k_adj_forward<1><<<blocks, 256, 0, a->stream>>>(f);
    else k_adj_forward<0><<<blocks, 256, 0, a->stream>>>(f);
    ACK(cudaGetLastError(), "k_adj_forward");
    cudaEventRecord(a->ph[1], a->stream);
    const unsigned gb = (unsigned)((G + 255) / 256);
    k_adj_loss<<<gb, 256, 0, a->stream>>>(a->dacc, a->target, (uint32_t)G, a->p.ticks, a->density, a->lambda,
                                          a->partial);
    k_adj_loss_final<<<1, 32, 0, a->stream>>>(a->partial, gb, (uint32_t)G, a->loss);
    ACK(cudaGetLastError(), "k_adj_loss");
    cudaEventRecord(a->ph[2], a->stream);
    if (d_density)
        ACK(cudaMemcpyAsync(d_density, a->density, sizeof(float) * G, cudaMemcpyDeviceToDevice, a->stream), "density");
    if (loss) ACK(cudaMemcpyAsync(loss, a->loss, sizeof(double), cudaMemcpyDeviceToHost, a->stream), "loss");
    int rc = check_status(a);
    if (rc != MSIM_OK) return rc;
    a->have_forward = true;
    a->last_mode = mode;
    a->have_sched = true;
    return MSIM_OK;
}

int msim_adj_backward(msim_adj* a, float* d_grad_speed, float* d_grad_factor) {
    msim::NvtxRange range("msim_adj_backward");
    if (!a) return fail(MSIM_ERR_INVALID, "NULL argument");
    if (!a->have_forward) return fail(MSIM_ERR_INVALID, "backward needs a forward first");
    cudaSetDevice(a->device);
    const size_t n = a->n;
    ACK(cudaMemsetAsync(a->carry, 0, sizeof(float2) * n, a->stream), "memset carry");
    ACK(cudaMemsetAsync(a->gspeed, 0, sizeof(double) * n, a->stream), "memset gspeed");
    AdjBack b{};
    b.f = fwd_args(a, 2u);  // the backward replays the last forward's schedule
    b.lambda = a->lambda;
    b.hist_pos = a->hist_pos;
    b.hist_head = a->hist_head;
    b.carry = a->carry;
    b.gspeed = a->gspeed;
    b.rec_road = a->rec_road;
    b.rec_val = a->rec_val;
    b.num_roads = a->R;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaEventRecord(a->ph[3], a->stream);
    for (int seg = (int)a->S - 1; seg >= 0; seg--) {
        b.seg = (uint32_t)seg;
        if (a->p.rng_kind == 1) k_adj_backward<1><<<blocks, 256, 0, a->stream>>>(b);
        else k_adj_backward<0><<<blocks, 256, 0, a->stream>>>(b);
        ACK(cudaGetLastError(), "k_adj_backward");
    }
    cudaEventRecord(a->ph[4], a->stream);
    // road gradients: stable sort of the records by road, then per-road sums in order
    const uint32_t total = (uint32_t)a->rec_count;
    ACK(cudaMemsetAsync(a->hist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, a->stream), "memset hist");
    k_adj_hist<<<1024, 256, 0, a->stream>>>(a->rec_road, a->rec_count, a->passes, a->hist);
    ACK(cudaGetLastError(), "k_adj_hist");
    ACK(cudaMemsetAsync(a->lookback, 0, sizeof(uint32_t) * (size_t)a->passes * a->rec_tiles * kRadix, a->stream),
        "memset lookback");
    ACK(cudaMemsetAsync(a->tickets, 0, sizeof(uint32_t) * kMaxPasses, a->stream), "memset tickets");
    for (uint32_t ps = 0; ps < a->passes; ps++) {
        const uint32_t* kin = ps == 0 ? a->rec_road : a->sk[(ps - 1) & 1];
        const uint32_t* vin = ps == 0 ? nullptr : a->sv[(ps - 1) & 1];
        ACK(launch_onesweep(a->stream, kin, vin, a->sk[ps & 1], a->sv[ps & 1], total, 8u * ps,
                            a->hist + ps * kRadix, a->lookback + (size_t)ps * a->rec_tiles * kRadix,
                            a->tickets + ps, a->err),
            "k_onesweep");
    }
    const uint32_t* sorted_key = a->sk[(a->passes - 1) & 1];
    const uint32_t* sorted_rec = a->sv[(a->passes - 1) & 1];
    ACK(launch_kstart(a->stream, sorted_key, total, a->kstart, a->R + 1), "k_kstart");
    k_adj_road_sum<<<(a->R + 255) / 256, 256, 0, a->stream>>>(a->kstart, sorted_rec, a->rec_val, a->R, total,
                                                              a->gfactor, d_grad_factor);
    ACK(cudaGetLastError(), "k_adj_road_sum");
    if (d_grad_speed) {
        k_adj_speed_out<<<blocks, 256, 0, a->stream>>>(a->gspeed, a->perm, a->n, d_grad_speed);
        ACK(cudaGetLastError(), "k_adj_speed_out");
    }
    cudaEventRecord(a->ph[5], a->stream);
    a->have_backward = true;
    return check_status(a);
}

int msim_adj_phase_times(msim_adj* a, float ms[4]) {
    if (!a || !ms) return fail(MSIM_ERR_INVALID, "NULL argument");
    if (!a->have_forward || !a->have_backward) return fail(MSIM_ERR_INVALID, "needs a forward and a backward first");
    cudaSetDevice(a->device);
    ACK(cudaStreamSynchronize(a->stream), "sync");
    ACK(cudaEventElapsedTime(&ms[0], a->ph[0], a->ph[1]), "cudaEventElapsedTime");
    ACK(cudaEventElapsedTime(&ms[1], a->ph[1], a->ph[2]), "cudaEventElapsedTime");
    ACK(cudaEventElapsedTime(&ms[2], a->ph[3], a->ph[4]), "cudaEventElapsedTime");
    ACK(cudaEventElapsedTime(&ms[3], a->ph[4], a->ph[5]), "cudaEventElapsedTime");
    return MSIM_OK;
}

int msim_adj_get_gradients_f64(msim_adj* a, double* grad_speed, double* grad_factor) {
    if (!a) return fail(MSIM_ERR_INVALID, "NULL argument");
    cudaSetDevice(a->device);
    ACK(cudaStreamSynchronize(a->stream), "sync");
    if (grad_speed) {
        std::vector<double> tmp(a->n);
        ACK(cudaMemcpy(tmp.data(), a->gspeed, sizeof(double) * a->n, cudaMemcpyDeviceToHost), "download");
        to_entity_order(a->hperm, tmp.data(), grad_speed);
    }
    if (grad_factor) ACK(cudaMemcpy(grad_factor, a->gfactor, sizeof(double) * a->R, cudaMemcpyDeviceToHost), "download");
    return MSIM_OK;
}

int msim_adj_get_schedule(msim_adj* a, uint32_t* words) {
    if (!a || !words) return fail(MSIM_ERR_INVALID, "NULL argument");
    if (!a->have_sched) return fail(MSIM_ERR_INVALID, "no recorded event schedule");
    cudaSetDevice(a->device);
    ACK(cudaStreamSynchronize(a->stream), "sync");
    std::vector<uint32_t> tmp((size_t)a->n * a->sched_words);
    ACK(cudaMemcpy(tmp.data(), a->sched, sizeof(uint32_t) * tmp.size(), cudaMemcpyDeviceToHost), "download schedule");
    to_entity_order(a->hperm, tmp.data(), words, a->sched_words);
    return MSIM_OK;
}

int msim_adj_timer_begin(msim_adj* a) {
    if (!a) return fail(MSIM_ERR_INVALID, "NULL argument");
    ACK(cudaEventRecord(a->t0, a->stream), "cudaEventRecord");
    return MSIM_OK;
}

int msim_adj_timer_end(msim_adj* a, float* ms) {
    if (!a || !ms) return fail(MSIM_ERR_INVALID, "NULL argument");
    ACK(cudaEventRecord(a->t1, a->stream), "cudaEventRecord");
    ACK(cudaEventSynchronize(a->t1), "cudaEventSynchronize");
    ACK(cudaEventElapsedTime(ms, a->t0, a->t1), "cudaEventElapsedTime");
    return MSIM_OK;
}

}  // extern "C"
