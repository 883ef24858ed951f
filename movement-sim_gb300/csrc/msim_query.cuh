// Key-start table and radius neighbour query (included by msim_kernels.cu inside
// its namespace).

// ---- key-start table ------------------------------------------------------------
// kstart[k] = first sorted position whose key is >= k, for every k in
// [0, num_keys]; kstart[num_keys] = n.  Keys >= num_keys (never produced by valid
// inputs) count as num_keys - 1.  A tile's run is [kstart[t << ybits],
// kstart[(t + 1) << ybits]); a band run inside it is two independent loads.
constexpr uint32_t kKstartWindow = 1024;  // table entries written by one warp

__device__ __forceinline__ uint32_t clamped_key(const uint32_t* __restrict__ sk, uint32_t q, uint32_t num_keys) {
    const uint32_t k = sk[q];
    return k < num_keys ? k : num_keys - 1u;
}

// One warp per window of kKstartWindow table entries [B, E): a 32-ary search finds
// the first position with key >= B, then the warp walks the positions 32 at a time.
// Position q owns the entries (key[q-1], key[q]] (clipped to the window); the
// lanes' entry counts are laid end to end (warp prefix sum) and written 32 at a
// time, each entry's owner found by a binary search over the prefix sums.  Every
// warp writes exactly its window, so no warp fills a long empty stretch of the key
// space alone.  For key spaces much smaller than n see k_kstart_search.
__global__ __launch_bounds__(256) void k_kstart(const uint32_t* __restrict__ sk, uint32_t n,
                                                uint32_t* __restrict__ kstart, uint32_t num_keys,
                                                const uint32_t* err) {
    constexpr uint32_t FULL = 0xffffffffu;
    if (index_failed(err)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t b64 = (uint64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kKstartWindow;
    if (b64 > num_keys) return;  // uniform per warp
    const uint32_t B = (uint32_t)b64;
    const uint32_t E = (uint32_t)(b64 + kKstartWindow < (uint64_t)num_keys + 1u ? b64 + kKstartWindow
                                                                                : (uint64_t)num_keys + 1u);
    // first position with key >= B: the answer stays in [lo, hi], key[hi] >= B or hi = n
    uint32_t lo = 0, hi = n;
    while (hi - lo > 32u) {
        const uint32_t step = (hi - lo + 31u) >> 5;
        const uint32_t q = min(lo + (lane + 1u) * step - 1u, hi - 1u);
        const uint32_t m = __ballot_sync(FULL, clamped_key(sk, q, num_keys) >= B);
        if (m == 0u) {  // the last probe is hi - 1
            lo = hi;
            break;
        }
        const uint32_t f = __ffs(m) - 1u;
        const uint32_t qf = min(lo + (f + 1u) * step - 1u, hi - 1u);
        lo = f ? min(lo + f * step - 1u, hi - 1u) + 1u : lo;
        hi = qf;
    }
    if (hi > lo) {
        const uint32_t q = lo + lane;
        const uint32_t m = __ballot_sync(FULL, q < hi && clamped_key(sk, q, num_keys) >= B);
        lo = m ? lo + __ffs(m) - 1u : hi;
    }
    uint32_t cursor = B;  // first entry of the window not yet written
    for (uint32_t q0 = lo; cursor < E; q0 += 32u) {
        const uint32_t q = q0 + lane;
        const uint32_t key = q < n ? clamped_key(sk, q, num_keys) : num_keys;  // n owns the tail up to num_keys
        const uint32_t prev = __shfl_up_sync(FULL, key, 1);
        const uint32_t a = lane ? prev + 1u : cursor;
        const uint32_t b = key < E - 1u ? key : E - 1u;
        const uint32_t len = b + 1u > a ? b + 1u - a : 0u;
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t excl = incl - len;
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t base = 0; base < total; base += 32u) {
            const uint32_t i = base + lane;
            uint32_t owner = 0;  // first lane whose inclusive prefix exceeds i
#pragma unroll
            for (uint32_t st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(FULL, incl, owner + st - 1u);
                if (v <= i) owner += st;
            }
            const uint32_t o_excl = __shfl_sync(FULL, excl, owner);
            const uint32_t o_a = __shfl_sync(FULL, a, owner);
            if (i < total) kstart[o_a + (i - o_excl)] = q0 + owner;
        }
        cursor = __shfl_sync(FULL, key, 31) + 1u;
    }
}

// One thread per position q in [0, n]: q owns the entries (key[q-1], key[q]] (q = n:
// up to num_keys).  Gaps of at most kGapDirect entries (almost all of them) are
// written by the thread itself; gaps up to kGapWarp entries by the whole warp (the
// lanes' gaps laid end to end, 32 coalesced entries per store); longer ones are cut
// into chunks of kGapChunk entries, appended to a list with one atomic per warp
// (disjoint entries, so the append order does not matter) and filled by
// k_kstart_fill.
constexpr uint32_t kGapDirect = 8;
constexpr uint32_t kGapWarp = 256;
constexpr uint32_t kGapChunk = 4096;

// Writes kstart[from + r] = value for r < len, for every lane of the warp (all lanes
// call it; a lane with nothing to write passes len = 0).
__device__ __forceinline__ void fill_key_gaps(uint32_t from, uint32_t len, uint32_t value, uint32_t lane,
                                              uint32_t* __restrict__ kstart, uint4* __restrict__ chunks,
                                              uint32_t* chunk_count, uint32_t chunk_cap) {
    constexpr uint32_t FULL = 0xffffffffu;
    if (len <= kGapDirect) {
        for (uint32_t r = 0; r < len; r++) kstart[from + r] = value;
    }
    // medium gaps: the warp writes them together
    const uint32_t wlen = len > kGapDirect && len <= kGapWarp ? len : 0u;
    if (__any_sync(FULL, wlen != 0u)) {
        uint32_t incl = wlen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t excl = incl - wlen;
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t base = 0; base < total; base += 32u) {
            const uint32_t i = base + lane;
            uint32_t owner = 0;
#pragma unroll
            for (uint32_t st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(FULL, incl, owner + st - 1u);
                if (v <= i) owner += st;
            }
            const uint32_t o_excl = __shfl_sync(FULL, excl, owner);
            const uint32_t o_from = __shfl_sync(FULL, from, owner);
            const uint32_t o_val = __shfl_sync(FULL, value, owner);
            if (i < total) kstart[o_from + (i - o_excl)] = o_val;
        }
    }
    // long gaps: chunks, one list append per warp
    const uint32_t m = len > kGapWarp ? (len + kGapChunk - 1u) / kGapChunk : 0u;
    if (__any_sync(FULL, m != 0u)) {
        uint32_t incl = m;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        uint32_t base = 0;
        if (lane == 31) base = atomicAdd(chunk_count, total);
        base = __shfl_sync(FULL, base, 31) + (incl - m);
        if (m) {
            if (base + m > chunk_cap) {  // unreachable: chunk_cap bounds every key space; stay correct anyway
                for (uint32_t r = 0; r < len; r++) kstart[from + r] = value;
            } else {
                for (uint32_t c = 0; c < m; c++) {
                    const uint32_t off = c * kGapChunk;
                    chunks[base + c] =
                        make_uint4(from + off, len - off < kGapChunk ? len - off : kGapChunk, value, 0u);
                }
            }
        }
    }
}

// Writes kstart[from + r] = value for r < len by one thread: directly up to kGapWarp
// entries, in kGapChunk-entry chunks appended to the list beyond that.
__device__ __forceinline__ void fill_run(uint32_t from, uint32_t len, uint32_t value, uint32_t* __restrict__ kstart,
                                         uint4* __restrict__ chunks, uint32_t* chunk_count, uint32_t chunk_cap) {
    if (len <= kGapWarp) {
        for (uint32_t r = 0; r < len; r++) kstart[from + r] = value;
        return;
    }
    const uint32_t m = (len + kGapChunk - 1u) / kGapChunk;
    const uint32_t base = atomicAdd(chunk_count, m);
    if (base + m > chunk_cap) {  // unreachable: chunk_cap bounds every key space; stay correct anyway
        for (uint32_t r = 0; r < len; r++) kstart[from + r] = value;
        return;
    }
    for (uint32_t c = 0; c < m; c++) {
        const uint32_t off = c * kGapChunk;
        chunks[base + c] = make_uint4(from + off, len - off < kGapChunk ? len - off : kGapChunk, value, 0u);
    }
}

__global__ __launch_bounds__(256) void k_kstart_pos(const uint32_t* __restrict__ sk, uint32_t n,
                                                    uint32_t* __restrict__ kstart, uint32_t num_keys,
                                                    uint4* __restrict__ chunks, uint32_t* chunk_count,
                                                    uint32_t chunk_cap, const uint32_t* __restrict__ sv,
                                                    const float2* __restrict__ pos, float2* __restrict__ sorted_pos,
                                                    const uint32_t* err) {
    chain_enter();
    if (index_failed(err)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (sorted_pos && q < n) {  // positions in sorted order, for the query's candidate reads
        const uint32_t slot = sv[q];
        sorted_pos[q] = slot < n ? pos[slot] : make_float2(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff));
    }
    uint32_t from = 0, len = 0;
    if (q <= n) {
        from = q ? clamped_key(sk, q - 1u, num_keys) + 1u : 0u;
        const uint32_t to = q < n ? clamped_key(sk, q, num_keys) : num_keys;  // inclusive
        len = to >= from ? to - from + 1u : 0u;
    }
    fill_key_gaps(from, len, q, lane, kstart, chunks, chunk_count, chunk_cap);
}

__global__ __launch_bounds__(256) void k_kstart_fill(const uint4* __restrict__ chunks,
                                                     const uint32_t* __restrict__ chunk_count, uint32_t chunk_cap,
                                                     uint32_t* __restrict__ kstart, const uint32_t* err) {
    chain_enter();
    if (index_failed(err)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t count = min(*chunk_count, chunk_cap);
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < count; c += warps) {
        const uint4 ch = chunks[c];
        for (uint32_t r = lane; r < ch.y; r += 32u) kstart[ch.x + r] = ch.z;
    }
}

// Chunk-list capacity that no key space can exceed: every chunked gap has more than
// kGapWarp entries, and adds at most one partial chunk.
inline uint32_t kstart_chunk_cap(uint64_t num_keys) {
    return (uint32_t)((num_keys + 1u) / (kGapWarp + 1u) + (num_keys + 1u) / kGapChunk + 2u);
}

// Positions in sorted order (NaN for a slot out of range), for the key-start paths
// that do not gather them on the way.
__global__ __launch_bounds__(256) void k_gather_pos(const uint32_t* __restrict__ sv, const float2* __restrict__ pos,
                                                    uint32_t n, float2* __restrict__ sorted_pos,
                                                    const uint32_t* err) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || index_failed(err)) return;
    const uint32_t slot = sv[q];
    sorted_pos[q] = slot < n ? pos[slot] : make_float2(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff));
}

// One thread per table entry, binary search over the sorted keys: for key spaces
// much smaller than the number of positions (many positions per key).
__global__ __launch_bounds__(256) void k_kstart_search(const uint32_t* __restrict__ sk, uint32_t n,
                                                       uint32_t* __restrict__ kstart, uint32_t num_keys,
                                                       const uint32_t* err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > num_keys || index_failed(err)) return;
    uint32_t lo = 0, hi = n;  // first position with clamped key >= k
    if (k == num_keys) {
        lo = n;
    } else {
        while (lo < hi) {
            const uint32_t mid = lo + ((hi - lo) >> 1);
            if (clamped_key(sk, mid, num_keys) < k) lo = mid + 1u;
            else hi = mid;
        }
    }
    kstart[k] = lo;
}

// ---- radius neighbour query ------------------------------------------------------
// A warp queries 32 consecutive sorted positions (mostly one or two tiles).  Each
// lane's box [pos - reach, pos + reach] covers one to four tiles (more only when the
// tile side is below 2 x reach); for every tile the lane reads the run of the y bands
// its box overlaps from the key-start table.  The warp lays all non-empty runs of its
// lanes end to end in a shared run list (flat start, start position, owner lane) and
// tests 32 (owner, candidate) pairs per iteration, so every lane is busy whatever the
// run lengths; the run of each pair comes from a bit mask of the runs that start in
// the current window of 32 pairs.  Every candidate is tested with the predicate of
// random_move.comp:551-562; candidate positions come from the sorted copy, read in
// runs.  A hit adds one to the owner's count and, for the first kRegKeep hits,
// keeps the candidate's sorted position; ids are looked up only for those.  An
// entity with more than kRegKeep neighbours redoes an exact pass into its output
// slots.  The predicate is symmetric (fl(a - b) = -fl(b - a)), so the pair count is
// half the sum of the counts, and a pair of entities of the same warp (most pairs:
// consecutive sorted entities share their band runs) is tested once, by the lower
// lane, which credits both.  Each warp writes its lists contiguously at
// warp * 32 * cap and adds its count sum to one of kPairBins counters; the kernel has
// no block-wide barrier.
constexpr uint32_t kRuns = 4;                  // runs per lane and round
constexpr uint32_t kWarpRuns = 32u * kRuns;    // run-list capacity of a warp

struct QueryShared {
    float2 me[kQueryThreads];
    uint32_t cnt[kQueryThreads];
    uint32_t keep[kRegKeep][kQueryThreads];    // sorted positions of the first kRegKeep hits
    uint32_t rq[kQueryThreads / 32][kWarpRuns];   // run start position minus its flat start
    uint32_t rfs[kQueryThreads / 32][kWarpRuns];  // flat start of the run
    uint32_t rown[kQueryThreads / 32][kWarpRuns]; // owner lane
};

template <bool LIST>
__device__ __forceinline__ void query_runs(const uint32_t (&lo_in)[kRuns], const uint32_t (&len_in)[kRuns],
                                           uint32_t lane, uint32_t warp, uint32_t pwarp, QueryShared& sh,
                                           const float2* __restrict__ sorted_pos, const TileGrid& g) {
    constexpr uint32_t FULL = 0xffffffffu;
    // A pair of entities of this warp is tested once, by the lower lane, which credits
    // both (the predicate is symmetric, and an in-range pair lies in both entities'
    // runs).  So a lane skips the warp's positions up to its own: a run that starts at
    // or after the warp's first position starts after the owner instead (a run that
    // starts before it is kept whole; the loop skips those positions).  At 16 M about
    // 4.7 of the 5.3 candidates of an entity lie in its own warp.
    uint32_t lo[kRuns], len[kRuns];
#pragma unroll
    for (uint32_t k = 0; k < kRuns; k++) {
        lo[k] = lo_in[k];
        len[k] = len_in[k];
        if (len[k] && lo[k] >= pwarp) {
            const uint32_t hi = lo[k] + len[k];
            const uint32_t from = lo[k] > pwarp + lane ? lo[k] : pwarp + lane + 1u;
            lo[k] = from;
            len[k] = hi > from ? hi - from : 0u;
        }
    }
    uint32_t flat = 0, nr = 0;
#pragma unroll
    for (uint32_t k = 0; k < kRuns; k++) {
        flat += len[k];
        nr += len[k] ? 1u : 0u;
    }
    uint32_t fi = flat, ri = nr;  // inclusive warp prefixes of candidates and runs
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t yf = __shfl_up_sync(FULL, fi, o);
        const uint32_t yr = __shfl_up_sync(FULL, ri, o);
        if (lane >= (uint32_t)o) {
            fi += yf;
            ri += yr;
        }
    }
    const uint32_t total = __shfl_sync(FULL, fi, 31);
    const uint32_t runs = __shfl_sync(FULL, ri, 31);
    uint32_t j = ri - nr, fs = fi - flat;
#pragma unroll
    for (uint32_t k = 0; k < kRuns; k++) {
        if (len[k]) {
            sh.rq[warp][j] = lo[k] - fs;
            sh.rfs[warp][j] = fs;
            sh.rown[warp][j] = lane;
            j++;
            fs += len[k];
        }
    }
    __syncwarp();  // the run list is visible to the whole warp
    uint32_t ra = 0;  // first run that starts at or after the current window
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t rr = ra + lane;
        const uint32_t off = (rr < runs ? sh.rfs[warp][rr] : 0xffffffffu) - base;
        const uint32_t marks = __reduce_or_sync(FULL, off < 32u ? (1u << off) : 0u);
        const uint32_t le = marks & (0xffffffffu >> (31u - lane));
        const uint32_t run = ra + (uint32_t)__popc(le) - 1u;  // le == 0: the run begun before the window
        ra += (uint32_t)__popc(marks);
        const uint32_t i = base + lane;
        if (i >= total) continue;
        const uint32_t q = sh.rq[warp][run] + i;
        const uint32_t owner = sh.rown[warp][run];
        const uint32_t other = q - pwarp;  // the candidate's lane when it is in this warp
        if (other <= owner) continue;      // the owner itself or a lower lane: tested from there
        const uint32_t ot = warp * 32u + owner;
        if (!in_range_fast(sorted_pos[q], sh.me[ot], g.radius, g.d2_limit)) continue;
        const uint32_t c = atomicAdd(&sh.cnt[ot], 1u);
        if (LIST && c < (uint32_t)kRegKeep) sh.keep[c][ot] = q;  // sorted position; the id comes later
        if (other < 32u) {  // a higher lane of this warp: the pair counts for it too
            const uint32_t om = warp * 32u + other;
            const uint32_t c2 = atomicAdd(&sh.cnt[om], 1u);
            if (LIST && c2 < (uint32_t)kRegKeep) sh.keep[c2][om] = pwarp + owner;
        }
    }
    __syncwarp();  // before the run list is rewritten
}

// 16 blocks (64 warps) per SM: at 40 registers (12 blocks) the symmetric pair loop
// gained nothing (0.435 against 0.437 ms at 16 M), at 32 it takes 0.395.
template <bool LIST>
__global__ __launch_bounds__(kQueryThreads, 16) void k_query(const uint32_t* __restrict__ kstart,
                                                         const uint32_t* __restrict__ sorted_slot,
                                                         const float2* __restrict__ sorted_pos,
                                                         const uint32_t* __restrict__ slot_id, TileGrid g,
                                                         uint32_t n, uint32_t cap, uint32_t* __restrict__ count_out,
                                                         uint32_t* __restrict__ list,
                                                         unsigned long long* __restrict__ pair_bins,
                                                         const uint32_t* err, uint32_t* __restrict__ count_by_id) {
    constexpr uint32_t FULL = 0xffffffffu;
    __shared__ QueryShared sh;
    if (index_failed(err)) return;  // uniform per block
    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31;
    const uint32_t warp = tid >> 5;
    const uint32_t p = blockIdx.x * kQueryThreads + tid;
    const uint32_t pwarp = p - lane;
    const bool valid = p < n;
    float2 me = make_float2(0.f, 0.f);
    uint32_t x0 = 1, x1 = 0, y0 = 1, y1 = 0;  // empty box for invalid lanes
    float ylo = 0.f, yhi = 0.f;
    if (valid) {
        me = sorted_pos[p];
        ylo = __fsub_rn(me.y, g.reach);
        yhi = __fadd_rn(me.y, g.reach);
        x0 = tile_coord(__fsub_rn(me.x, g.reach), g.inv_cell, g.tiles_x);
        x1 = tile_coord(__fadd_rn(me.x, g.reach), g.inv_cell, g.tiles_x);
        y0 = tile_coord(ylo, g.inv_cell, g.tiles_y);
        y1 = tile_coord(yhi, g.inv_cell, g.tiles_y);
    }
    sh.me[tid] = me;
    sh.cnt[tid] = 0u;
    const uint32_t nx = x1 >= x0 ? x1 - x0 + 1u : 0u, ny = y1 >= y0 ? y1 - y0 + 1u : 0u;
    if (__all_sync(FULL, nx <= 2u && ny <= 2u)) {
        // at most 2 x 2 tiles (always when the tile side is at least 2 x reach): the
        // tiles' Morton codes by increments; the row y0 runs from the lower box edge's
        // band up (to the last band when the box reaches row y1), row y1 from band 0
        const uint32_t top = (1u << g.ybits) - 1u;
        const uint32_t b_lo = g.ybits ? y_band(g, ylo, y0) : 0u;
        const uint32_t b_hi = g.ybits ? y_band(g, yhi, y1) : 0u;
        const uint32_t m00 = morton2_tile(x0, y0);
        const uint32_t m10 = morton_inc_x(m00);
        const uint32_t tiles[kRuns] = {m00, m10, morton_inc_y(m00), morton_inc_y(m10)};
        const bool have[kRuns] = {nx >= 1u && ny >= 1u, nx == 2u && ny >= 1u, nx >= 1u && ny == 2u,
                                  nx == 2u && ny == 2u};
        uint32_t lo[kRuns], len[kRuns];
#pragma unroll
        for (uint32_t k = 0; k < kRuns; k++) {
            lo[k] = 0u;
            len[k] = 0u;
            if (__any_sync(FULL, have[k]) && have[k]) {
                const uint32_t t = tiles[k] << g.ybits;
                const uint32_t bl = k < 2u ? b_lo : 0u;
                const uint32_t bh = k < 2u ? (ny == 2u ? top : b_hi) : b_hi;
                lo[k] = kstart[t | bl];
                uint32_t hi = kstart[(t | bh) + 1u];
                if (hi > n) hi = n;
                len[k] = hi > lo[k] ? hi - lo[k] : 0u;
            }
        }
        query_runs<LIST>(lo, len, lane, warp, pwarp, sh, sorted_pos, g);
    } else {
        // general boxes (tile side below 2 x reach): kRuns tiles per round
        const uint32_t nslots = nx * ny;
        const uint32_t max_slots = __reduce_max_sync(FULL, nslots);
#pragma unroll 1
        for (uint32_t j0 = 0; j0 < max_slots; j0 += kRuns) {
            uint32_t lo[kRuns], len[kRuns];
#pragma unroll
            for (uint32_t k = 0; k < kRuns; k++) {
                const uint32_t j = j0 + k;
                lo[k] = 0u;
                len[k] = 0u;
                if (j < nslots) {
                    const uint32_t jy = j / nx;
                    const uint32_t tx = x0 + (j - jy * nx), ty = y0 + jy;
                    const uint32_t t = morton2(tx, ty) << g.ybits;
                    const uint32_t b0 = g.ybits ? y_band(g, ylo, ty) : 0u;
                    const uint32_t b1 = g.ybits ? y_band(g, yhi, ty) : 0u;
                    lo[k] = kstart[t | b0];
                    uint32_t hi = kstart[(t | b1) + 1u];
                    if (hi > n) hi = n;
                    len[k] = hi > lo[k] ? hi - lo[k] : 0u;
                }
            }
            query_runs<LIST>(lo, len, lane, warp, pwarp, sh, sorted_pos, g);
        }
    }
    __syncwarp();
    const uint32_t count = valid ? sh.cnt[tid] : 0u;
    if (valid) {
        count_out[p] = count;
        // slots that hold their own entity: the count also goes straight to its id's
        // place (the host tick downloads these, with no export pass after the query)
        if (count_by_id) count_by_id[sorted_slot[p]] = count;
    }
    const uint32_t warp_sum = __reduce_add_sync(FULL, count);  // every pair is seen from both ends
    if (lane == 0 && warp_sum) atomicAdd(&pair_bins[(p >> 5) & (kPairBins - 1u)], (unsigned long long)warp_sum);
    if (LIST) {
        const uint32_t kept = count < cap ? count : cap;
        uint32_t incl = kept;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        uint32_t* out = list + (size_t)(p >> 5) * 32u * cap + (incl - kept);
        // the warp's largest kept list bounds the (warp-uniform) id fetch and insertion
        const uint32_t wmax = __reduce_max_sync(FULL, count <= (uint32_t)kRegKeep ? count : 0u);
        if (count <= (uint32_t)kRegKeep) {  // every neighbour is kept: ids, sort, write
            uint32_t id[kRegKeep];
#pragma unroll
            for (int i = 0; i < kRegKeep; i++) {  // all fetches of a lane in flight together
                id[i] = 0xffffffffu;
                if ((uint32_t)i < wmax) {
                    const uint32_t s2 = (uint32_t)i < count ? sorted_slot[sh.keep[i][tid]] : n;
                    id[i] = s2 < n ? (slot_id ? slot_id[s2] : s2) : 0xffffffffu;  // NULL: slot = id
                }
            }
            uint32_t keep[kRegKeep];  // ascending; unused slots hold 0xffffffff
#pragma unroll
            for (int i = 0; i < kRegKeep; i++) keep[i] = 0xffffffffu;
#pragma unroll
            for (int i = 0; i < kRegKeep; i++) {
                if ((uint32_t)i >= wmax) continue;  // uniform
                // keep[0..i) is sorted and slot i is free: insert there and sink it, i
                // compare-exchanges (w (w - 1) / 2 in all for a warp's largest list w)
                keep[i] = id[i];
#pragma unroll
                for (int j = i; j > 0; j--) {
                    const uint32_t lo = min(keep[j - 1], keep[j]), hi = max(keep[j - 1], keep[j]);
                    keep[j - 1] = lo;
                    keep[j] = hi;
                }
            }
#pragma unroll
            for (int i = 0; i < kRegKeep; i++) {
                if ((uint32_t)i >= wmax) break;  // uniform
                if ((uint32_t)i < kept) out[i] = keep[i];
            }
        } else {
            list_overflow(sorted_slot, sorted_pos, slot_id, kstart, g, n, p, cap, out);
        }
    }
}
