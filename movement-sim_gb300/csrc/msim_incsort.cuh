// Incremental index update (included by msim_kernels.cu inside its namespace).
//
// Between two neighbour ticks an entity keeps its sort key unless it crosses a y
// band or a tile: a few per cent of the entities per tick.  Instead of sorting all
// keys again, the previous sorted order P (slots) with its keys PK is split into
//   A: the entries whose key is unchanged, in P's order - still sorted, and
//   B: the entries whose key changed (with the new key), in P's order;
// B alone is radix-sorted (stable), and A and B are merged (A first on equal keys).
// The merge writes the new sorted keys and slots, the key-start table and the
// positions in sorted order in the same pass.  The result is a valid key order; the
// order of equal keys differs from a full stable sort, which nothing observable
// depends on (neighbour sets are sets, lists are sorted by id).

constexpr uint32_t kMarkThreads = 256;
constexpr uint32_t kMarkPer = 16;                           // rows of a tile (entries per thread)
constexpr uint32_t kMarkTile = kMarkThreads * kMarkPer;     // 4096
constexpr uint32_t kMergeThreads = 256;
constexpr uint32_t kMergeTile = 1024;                       // output positions per block (16 M:
                                                            // 0.177 ms per merge, 0.190 with 2048)
// look-back word of k_mark: flag (bits 62-63) | A count (bits 31-61) | B count (bits 0-30)
constexpr unsigned long long kMarkAgg = 1ull << 62;
constexpr unsigned long long kMarkPrefix = 2ull << 62;
constexpr unsigned long long kMarkField = (1ull << 31) - 1ull;

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Splits P into A and B (stable), counts B's radix digits, and (last tile) writes
// counts[0] = |A|, counts[1] = |B|.  A tile of 4096 positions is read row by row
// (row r = 256 consecutive positions, coalesced); each entry's rank inside its list
// comes from per-row ballots and a scan of the per-(row, warp) counts, so the tile's
// A and B entries are staged in q order in shared memory and written out coalesced.
// Tiles are taken in ticket order and find their output offsets by a warp-wide
// decoupled look-back (32 predecessors per round of loads).  identity: P[q] = q
// (right after the state was re-ordered).  Five blocks per SM (48 registers): the
// split waits on its barriers and look-back, so more resident tiles hide that
// (measured at 16 M: 0.114 ms against 0.120 with four blocks, 0.118 with six).
__global__ __launch_bounds__(kMarkThreads, 5) void k_mark(const uint32_t* __restrict__ P, uint32_t identity,
                                                       const uint32_t* __restrict__ PK,
                                                       const uint32_t* __restrict__ NK, uint32_t n, uint32_t passes,
                                                       uint32_t* __restrict__ a_key, uint32_t* __restrict__ a_val,
                                                       uint32_t* __restrict__ b_key, uint32_t* __restrict__ b_val,
                                                       uint32_t* hist, unsigned long long* lookback, uint32_t* ticket,
                                                       uint32_t num_tiles, uint32_t* counts, uint32_t* err,
                                                       unsigned long long* changed_total, uint32_t spin_limit) {
    constexpr uint32_t FULL = 0xffffffffu;
    constexpr uint32_t NW = kMarkThreads / 32;
    __shared__ uint32_t s_key[kMarkTile], s_val[kMarkTile];  // A entries, then B entries, in q order
    __shared__ uint32_t s_hist[kMaxPasses * kRadix];
    __shared__ uint32_t s_off[kMarkPer * NW + 1];            // exclusive A counts before (row, warp)
    __shared__ uint32_t s_bal[kMarkPer * NW];                // the (row, warp) ballots of unchanged keys
    __shared__ uint32_t s_tile, s_pa, s_pb;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    chain_enter();
    if (index_failed(err)) return;  // an earlier wait gave up: the previous order is incomplete
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    for (uint32_t i = tid; i < passes * kRadix; i += kMarkThreads) s_hist[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= num_tiles) return;  // only when the ticket did not start at zero; uniform per block
    const uint32_t base = tile * kMarkTile;
    const uint32_t lt = lanemask_lt();
    // the row ballots go to shared memory (each lane's rank and A/B side come back from
    // them at staging), so a thread holds only its keys and slots: fewer registers
    uint32_t kn[kMarkPer], sl[kMarkPer];
#pragma unroll
    for (uint32_t r = 0; r < kMarkPer; r++) {
        const uint32_t q = base + r * kMarkThreads + tid;
        sl[r] = 0u;
        kn[r] = 0u;
        bool u = false;
        if (q < n) {
            sl[r] = identity ? q : P[q];
            kn[r] = NK[sl[r] < n ? sl[r] : 0u];
            u = kn[r] == PK[q];
        }
        const unsigned bal = __ballot_sync(FULL, u);
        if (lane == 0) {
            s_off[r * NW + warp] = (uint32_t)__popc(bal);
            s_bal[r * NW + warp] = bal;
        }
    }
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the kMarkPer * NW counts, in (row, warp) order
        constexpr uint32_t E = kMarkPer * NW / 32;  // counts per lane
        static_assert(kMarkPer * NW % 32 == 0, "whole counts per lane");
        uint32_t v[E], sum = 0u;
#pragma unroll
        for (uint32_t k = 0; k < E; k++) {
            v[k] = s_off[lane * E + k];
            sum += v[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (uint32_t k = 0; k < E; k++) {
            s_off[lane * E + k] = run;
            run += v[k];
        }
        if (lane == 31) {
            s_off[kMarkPer * NW] = run;
            // publish the tile's counts at once: later tiles' look-back need not wait
            // for this tile's staging
            const uint32_t ta = run, tb = (n > base ? min(n - base, kMarkTile) : 0u) - run;
            st_relaxed64(lookback + tile,
                         (tile == 0 ? kMarkPrefix : kMarkAgg) | ((unsigned long long)ta << 31) | tb);
        }
    }
    __syncthreads();
    const uint32_t valid_in_tile = n > base ? min(n - base, kMarkTile) : 0u;
    const uint32_t tot_a = s_off[kMarkPer * NW], tot_b = valid_in_tile - tot_a;
#pragma unroll
    for (uint32_t r = 0; r < kMarkPer; r++) {  // stage in shared memory: A at [0, tot_a), B after
        const uint32_t i = r * kMarkThreads + tid;  // linear index in the tile = q - base
        if (i >= valid_in_tile) continue;
        const unsigned bal = s_bal[r * NW + warp];
        const bool u = (bal >> lane) & 1u;
        const uint32_t ra = s_off[r * NW + warp] + (uint32_t)__popc(bal & lt);  // A entries before it
        const uint32_t dst = u ? ra : tot_a + (i - ra);
        if (dst < kMarkTile) {
            s_key[dst] = kn[r];
            s_val[dst] = sl[r];
        }
        if (!u)
            for (uint32_t ps = 0; ps < passes; ps++)
                atomicAdd(&s_hist[ps * kRadix + ((kn[r] >> (8u * ps)) & 0xffu)], 1u);
    }
    if (warp == 0) {  // look back (the counts were published after the scan)
        uint32_t ea = 0u, eb = 0u;
        if (tile > 0) {
            int32_t j = (int32_t)tile - 1;
            uint32_t spins = 0u;
            for (;;) {
                const int32_t idx = j - (int32_t)lane;
                const unsigned long long w = idx >= 0 ? ld_relaxed64(lookback + idx) : kMarkPrefix;
                const uint32_t flag = (uint32_t)(w >> 62);
                const unsigned prefix = __ballot_sync(FULL, flag == 2u);
                const unsigned not_ready = __ballot_sync(FULL, flag == 0u);
                const uint32_t first = prefix ? (uint32_t)(__ffs(prefix) - 1) : 32u;
                const unsigned needed = first == 32u ? FULL : (0xffffffffu >> (31u - first));
                if (not_ready & needed) {  // a predecessor has not published: poll again
                    if (++spins > spin_limit) {
                        if (lane == 0) atomicOr(err, kErrTimeout);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                const bool take = lane <= first;
                ea += __reduce_add_sync(FULL, take ? (uint32_t)((w >> 31) & kMarkField) : 0u);
                eb += __reduce_add_sync(FULL, take ? (uint32_t)(w & kMarkField) : 0u);
                if (first < 32u) break;
                j -= 32;
            }
            if (lane == 0)
                st_relaxed64(lookback + tile, kMarkPrefix | ((unsigned long long)(ea + tot_a) << 31) | (eb + tot_b));
        }
        if (lane == 0) {
            s_pa = ea;
            s_pb = eb;
            if (tile == num_tiles - 1) {
                counts[0] = ea + tot_a;
                counts[1] = eb + tot_b;
                if (changed_total) atomicAdd(changed_total, (unsigned long long)(eb + tot_b));
            }
        }
    }
    __syncthreads();
    const uint32_t pa = s_pa, pb = s_pb;
    for (uint32_t i = tid; i < valid_in_tile; i += kMarkThreads) {  // coalesced runs out
        if (i < tot_a) {
            if (pa + i < n) {
                a_key[pa + i] = s_key[i];
                a_val[pa + i] = s_val[i];
            }
        } else if (pb + (i - tot_a) < n) {
            b_key[pb + (i - tot_a)] = s_key[i];
            b_val[pb + (i - tot_a)] = s_val[i];
        }
    }
    for (uint32_t i = tid; i < passes * kRadix; i += kMarkThreads) {
        const uint32_t v = s_hist[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Merge path: split[t] = number of A entries among the first min(t * kMergeTile, n)
// entries of the merge (A first on equal keys): the first i in [max(0, d - |B|),
// min(d, |A|)] with A[i] > B[d - 1 - i] (or the upper end).  One warp per tile
// boundary, 32-ary search: 32 probes per round, so about five rounds of dependent
// loads at 16 M entries instead of 24 for a binary search.
__global__ __launch_bounds__(256) void k_merge_path(const uint32_t* __restrict__ a_key,
                                                    const uint32_t* __restrict__ b_key,
                                                    const uint32_t* __restrict__ counts, uint32_t n,
                                                    uint32_t boundaries, uint32_t* __restrict__ split,
                                                    const uint32_t* err) {
    constexpr uint32_t FULL = 0xffffffffu;
    chain_enter();
    if (index_failed(err)) return;
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (t >= boundaries) return;  // uniform per warp
    const uint32_t na = counts[0], nb = counts[1];
    const uint32_t d = min(t * kMergeTile, n);
    // the answer stays in [lo, hi]; A[hi] > B[d - 1 - hi] or hi is the upper end
    uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
    while (hi - lo > 32u) {
        const uint32_t step = (hi - lo + 31u) >> 5;
        const uint32_t i = min(lo + (lane + 1u) * step - 1u, hi - 1u);
        const unsigned m = __ballot_sync(FULL, a_key[i] > b_key[d - 1u - i]);
        if (m == 0u) {  // the last probe is hi - 1: every index below hi belongs to the prefix
            lo = hi;
            break;
        }
        const uint32_t f = __ffs(m) - 1u;
        const uint32_t xf = min(lo + (f + 1u) * step - 1u, hi - 1u);
        lo = f ? min(lo + f * step - 1u, hi - 1u) + 1u : lo;
        hi = xf;
    }
    if (hi > lo) {
        const uint32_t i = lo + lane;
        const unsigned m = __ballot_sync(FULL, i < hi && a_key[i] > b_key[d - 1u - i]);
        lo = m ? lo + __ffs(m) - 1u : hi;
    }
    if (lane == 0) split[t] = lo;
}

// Merges tile t of the output: A entries [split[t], split[t+1]) and the matching B
// entries, in shared memory (ranks by binary search in the other segment), then
// writes the sorted keys and slots, the positions in sorted order and the key-start
// entries owned by each thread's consecutive positions (one walk per thread, fill_run).
// 8 blocks per SM (32 registers): 0.158 ms at 16 M against 0.173 at the 40 registers
// the compiler picks alone (6 blocks).
__global__ __launch_bounds__(kMergeThreads, 8) void k_merge(
    const uint32_t* __restrict__ a_key, const uint32_t* __restrict__ a_val, const uint32_t* __restrict__ b_key,
    const uint32_t* __restrict__ b_val, const uint32_t* __restrict__ counts, const uint32_t* __restrict__ split,
    uint32_t n, uint32_t* __restrict__ out_key, uint32_t* __restrict__ out_val, const float2* __restrict__ pos,
    float2* __restrict__ sorted_pos, uint32_t* __restrict__ kstart, uint32_t num_keys, uint4* __restrict__ chunks,
    uint32_t* chunk_count, uint32_t chunk_cap, uint32_t* err, uint32_t* __restrict__ rank) {
    __shared__ uint32_t s_ink[kMergeTile], s_inv[kMergeTile];    // A segment, then B segment
    __shared__ uint32_t s_outk[kMergeTile], s_outv[kMergeTile];
    __shared__ uint32_t s_prev;  // clamped key of the entry before the tile
    chain_enter();
    if (index_failed(err)) return;
    const uint32_t tid = threadIdx.x;
    const uint32_t na_all = counts[0], nb_all = counts[1];
    if (na_all + nb_all != n) {  // unreachable unless the split look-back gave up
        if (tid == 0) atomicOr(err, kErrOob);
        return;
    }
    const uint32_t d0 = blockIdx.x * kMergeTile;
    if (d0 >= n) return;
    const uint32_t d1 = min(d0 + kMergeTile, n);
    const uint32_t a0 = min(split[blockIdx.x], na_all), a1 = min(split[blockIdx.x + 1], na_all);
    const uint32_t b0 = d0 - a0, b1 = d1 - a1;
    const uint32_t na = a1 > a0 ? a1 - a0 : 0u;
    const uint32_t nb = b1 > b0 && b1 <= nb_all ? b1 - b0 : 0u;
    if (na + nb != d1 - d0) {  // unreachable: the splits come from the same counts
        if (tid == 0) atomicOr(err, kErrOob);
        return;
    }
    if (tid == 0) {
        uint32_t prev = 0xffffffffu;  // none before position 0
        if (d0 > 0) {
            const uint32_t ka = a0 > 0 ? a_key[a0 - 1u] : 0u;
            const uint32_t kb = b0 > 0 && b0 <= nb_all ? b_key[b0 - 1u] : 0u;
            prev = max(ka, kb);
            prev = prev < num_keys ? prev : num_keys - 1u;
        }
        s_prev = prev;
    }
    constexpr uint32_t kPer = kMergeTile / kMergeThreads;
    {  // every load of a thread is in flight before the first shared store
        uint32_t ik[kPer], iv[kPer];
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = k * kMergeThreads + tid;
            ik[k] = 0u;
            iv[k] = 0u;
            if (i < na) {
                ik[k] = a_key[a0 + i];
                iv[k] = a_val[a0 + i];
            } else if (i < na + nb) {
                ik[k] = b_key[b0 + (i - na)];
                iv[k] = b_val[b0 + (i - na)];
            }
        }
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = k * kMergeThreads + tid;
            if (i < na + nb) {
                s_ink[i] = ik[k];
                s_inv[i] = iv[k];
            }
        }
    }
    __syncthreads();
    for (uint32_t i = tid; i < na + nb; i += kMergeThreads) {
        const uint32_t k = s_ink[i];
        uint32_t r;
        if (i < na) {  // B entries before it: keys < k
            uint32_t lo = 0, hi = nb;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_ink[na + mid] < k) lo = mid + 1u;
                else hi = mid;
            }
            r = i + lo;
        } else {  // A entries before it: keys <= k
            uint32_t lo = 0, hi = na;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_ink[mid] <= k) lo = mid + 1u;
                else hi = mid;
            }
            r = (i - na) + lo;
        }
        if (r < kMergeTile) {
            s_outk[r] = k;
            s_outv[r] = s_inv[i];
        }
    }
    __syncthreads();
    const uint32_t cnt = d1 - d0;
    const uint32_t prev_tile = s_prev;
    if (sorted_pos) {
        float2 gp[kPer];  // the positions of a thread's outputs, gathered together
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = k * kMergeThreads + tid;
            const uint32_t slot = i < cnt ? s_outv[i] : n;
            gp[k] = slot < n ? pos[slot] : make_float2(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff));
        }
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {  // sorted keys, slots and positions: coalesced rows
            const uint32_t i = k * kMergeThreads + tid;
            if (i < cnt) {
                const uint32_t p = d0 + i;
                out_key[p] = s_outk[i];
                out_val[p] = s_outv[i];
                sorted_pos[p] = gp[k];
            }
        }
    } else {  // an index whose query reads the positions from elsewhere
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = k * kMergeThreads + tid;
            if (i < cnt) {
                out_key[d0 + i] = s_outk[i];
                out_val[d0 + i] = s_outv[i];
            }
        }
    }
    if (rank) {  // sorted position of every slot (ticks that reuse this index place their moves)
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = k * kMergeThreads + tid;
            if (i < cnt && s_outv[i] < n) rank[s_outv[i]] = d0 + i;
        }
    }
    // Key-start entries: position p owns the entries (key[p-1], key[p]], so the kPer
    // consecutive positions [tid * kPer, tid * kPer + kPer) of a thread own one
    // contiguous stretch of the table, written in one walk (about kPer entries at
    // the workloads' densities; a walk costs a few instructions per entry where a
    // per-position fill ran a warp-wide loop to the longest gap of each row).  Gaps
    // longer than kGapWarp entries go to the chunk list (k_kstart_fill).
    const uint32_t i0 = tid * kPer;
    if (i0 < cnt) {
        const uint32_t kp = i0 ? s_outk[i0 - 1u] : prev_tile;
        uint32_t e = d0 + i0 == 0 ? 0u : (kp < num_keys ? kp : num_keys - 1u) + 1u;  // first entry not yet owned
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint32_t i = i0 + k;
            if (i >= cnt) break;
            const uint32_t key = s_outk[i];
            const uint32_t kc = key < num_keys ? key : num_keys - 1u;
            if (kc >= e) {
                fill_run(e, kc - e + 1u, d0 + i, kstart, chunks, chunk_count, chunk_cap);
                e = kc + 1u;
            }
        }
    }
    if (d1 == n && tid == 0) {  // the tail (key[n-1], num_keys] belongs to n
        const uint32_t kl = s_outk[cnt - 1u];
        const uint32_t from = (kl < num_keys ? kl : num_keys - 1u) + 1u;
        fill_run(from, num_keys + 1u - from, n, kstart, chunks, chunk_count, chunk_cap);
    }
}
