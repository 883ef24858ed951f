/*
 * msim_oracle.c - CPU oracle for the movement-sim per-tick path.
 *
 * TEST INFRASTRUCTURE ONLY (tests, smoke check, bench.py CPU baseline).  Built
 * with -ffp-contract=off and without fast-math so every float operation is one
 * IEEE-754 binary32 operation in source order, as the semantics fixed for the
 * CUDA path require (no FMA contraction, correctly rounded sqrt and divide).
 *
 * Each function cites the reference lines it restates
 * (src/sim/shader/random_move.comp unless noted).
 */
#include "msim_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define HEAD_TO_END 0x80000000u
#define HEAD_ROAD 0x7fffffffu

/* ---- RNG ---------------------------------------------------------------- */

/* random_move.comp:725-736: t = w; s = x; w = z; z = y; y = s;
 * t ^= t << 11; t ^= t >> 8; x = t ^ s ^ (s >> 19); return x. */
uint32_t oracle_xs128_next(uint32_t s[4]) {
    uint32_t t = s[3];
    uint32_t x = s[0];
    s[3] = s[2];
    s[2] = s[1];
    s[1] = x;
    t ^= t << 11;
    t ^= t >> 8;
    s[0] = t ^ x ^ (x >> 19);
    return s[0];
}

/* PCG-XSH-RR: O'Neill, "PCG: A Family of Simple Fast Space-Efficient
 * Statistically Good Algorithms for Random Number Generation" (2014). */
uint32_t oracle_pcg32_next(uint32_t s[4]) {
    uint64_t old = (uint64_t)s[0] | ((uint64_t)s[1] << 32);
    uint64_t inc = (uint64_t)s[2] | ((uint64_t)s[3] << 32);
    uint64_t nxt = old * 6364136223846793005ULL + inc;
    s[0] = (uint32_t)nxt;
    s[1] = (uint32_t)(nxt >> 32);
    uint32_t xorshifted = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

void oracle_pcg32_seed(uint32_t s[4], uint64_t initstate, uint64_t initseq) {
    uint64_t inc = (initseq << 1) | 1u;
    s[0] = 0;
    s[1] = 0;
    s[2] = (uint32_t)inc;
    s[3] = (uint32_t)(inc >> 32);
    (void)oracle_pcg32_next(s);
    uint64_t st = ((uint64_t)s[0] | ((uint64_t)s[1] << 32)) + initstate;
    s[0] = (uint32_t)st;
    s[1] = (uint32_t)(st >> 32);
    (void)oracle_pcg32_next(s);
}

static inline uint32_t rng_next(uint32_t kind, uint32_t s[4]) {
    return kind == 1 ? oracle_pcg32_next(s) : oracle_xs128_next(s);
}

/* random_move.comp:738-741: float(u) * (1.0 / 4294967296.0).  The conversion
 * rounds to nearest even; the scale by 2^-32 is exact; u >= 2^32 - 128 gives 1.0. */
float oracle_next_float(uint32_t u) {
    volatile float f = (float)u;
    return f * 2.3283064365386962890625e-10f;
}

/* random_move.comp:743-746: uint(ceil(float(min) + f * float(max - min + 1))) - 1,
 * the product and the sum each rounded separately. */
uint32_t oracle_ranged(uint32_t u, uint32_t lo, uint32_t hi) {
    float f = oracle_next_float(u);
    float span = (float)(hi - lo + 1u);
    float prod = f * span;
    float v = (float)lo + prod;
    return (uint32_t)ceilf(v) - 1u;
}

void oracle_rng_seq(uint32_t kind, uint32_t s[4], uint32_t n, uint32_t* out) {
    for (uint32_t i = 0; i < n; i++) out[i] = rng_next(kind, s);
}

/* ---- deterministic draws -------------------------------------------------- */

/* splitmix64 output function (Steele, Lea, Flood 2014). */
uint64_t oracle_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

uint64_t oracle_draw(uint64_t seed, uint64_t stream, uint64_t i) {
    return oracle_splitmix64(oracle_splitmix64(seed + 0x632BE59BD9B4E019ULL * stream) + i);
}

static inline float unit24(uint64_t d) { return (float)(uint32_t)(d >> 40) * 5.9604644775390625e-8f; }

/* Simulator.cpp:114-129 (road uniform, target = road end, pos = road start) with
 * deterministic draws instead of std::random_device (Entity.cpp:44-49,
 * Map.cpp:152-157).  Streams: 1 road, 2 fraction, 3 speed, 4/5 rng. */
void oracle_init_entities(uint32_t num_roads, const float* road_pos, uint32_t n, uint32_t rng_kind,
                          uint64_t seed, uint32_t placement, float speed_min, float speed_max,
                          float* pos, uint32_t* heading, uint32_t* rng, float* speed) {
    for (uint32_t i = 0; i < n; i++) {
        uint64_t d_road = oracle_draw(seed, 1, i);
        uint32_t r = (uint32_t)(((d_road >> 32) * (uint64_t)num_roads) >> 32);
        const float* rp = road_pos + 4ull * r;
        float px = rp[0], py = rp[1];
        if (placement == 1) {
            float u = unit24(oracle_draw(seed, 2, i));
            float ex = rp[2] - rp[0];
            float ey = rp[3] - rp[1];
            float ox = u * ex;
            float oy = u * ey;
            px = rp[0] + ox;
            py = rp[1] + oy;
        }
        pos[2ull * i] = px;
        pos[2ull * i + 1] = py;
        heading[i] = r | HEAD_TO_END;
        float v = unit24(oracle_draw(seed, 3, i));
        float span = speed_max - speed_min;
        float sv = v * span;
        speed[i] = speed_min + sv;
        uint64_t a = oracle_draw(seed, 4, i);
        uint64_t b = oracle_draw(seed, 5, i);
        uint32_t* s = rng + 4ull * i;
        if (rng_kind == 1) {
            oracle_pcg32_seed(s, a, b);
        } else {
            s[0] = (uint32_t)a;
            s[1] = (uint32_t)(a >> 32);
            s[2] = (uint32_t)b;
            s[3] = (uint32_t)(b >> 32);
            if ((s[0] | s[1] | s[2] | s[3]) == 0) s[0] = 1;
        }
    }
}

/* ---- move step -------------------------------------------------------------- */

typedef struct {
    uint32_t num_roads;
    const float* road_pos;
    const uint32_t* road_conn;
    uint32_t num_conn;
    const uint32_t* conn;
    uint32_t rng_kind;
    float dt;
    const float* factor;
    uint32_t ticks;
    float* pos;
    uint32_t* heading;
    uint32_t* rng;
    const float* speed;
    uint32_t begin, end;
} step_job;

/* connections[] read with the pad rule: index num_conn reads the last entry. */
static inline uint32_t conn_at(const step_job* j, uint32_t k) {
    return k < j->num_conn ? j->conn[k] : j->conn[j->num_conn - 1];
}

/* One tick for entity i:
 *   main move branch   random_move.comp:869-874
 *   update_direction   :830-839  (d = target - pos, len = length(d), dir = d/len*SPEED)
 *   move               :841-852  (distance > SPEED ? pos + dir : snap + new_target)
 *   new_target         :778-828
 * SPEED (:750) becomes step = (speed * factor[road]) * dt; 1.4 * 1 * 1 = SPEED. */
static void step_entity(const step_job* j, uint32_t i) {
    float px = j->pos[2ull * i], py = j->pos[2ull * i + 1];
    uint32_t h = j->heading[i];
    uint32_t r = h & HEAD_ROAD;
    uint32_t to_end = h >> 31;
    const float* rp = j->road_pos + 4ull * r;
    float tx = to_end ? rp[2] : rp[0];
    float ty = to_end ? rp[3] : rp[1];
    float f = j->factor ? j->factor[r] : 1.0f;
    float sf = j->speed[i] * f;
    float step = sf * j->dt;
    float dx = tx - px;
    float dy = ty - py;
    float dx2 = dx * dx;
    float dy2 = dy * dy;
    float len = sqrtf(dx2 + dy2);
    if (len > step) {
        float nx = dx / len;
        float ny = dy / len;
        float mx = nx * step;
        float my = ny * step;
        j->pos[2ull * i] = px + mx;
        j->pos[2ull * i + 1] = py + my;
        return;
    }
    /* snap to the target, then new_target */
    j->pos[2ull * i] = tx;
    j->pos[2ull * i + 1] = ty;
    const uint32_t* rc = j->road_conn + 4ull * r;
    uint32_t cidx, ccnt;
    if (!to_end) { /* target == curRoad.start.pos (:786-793) */
        cidx = rc[0];
        ccnt = rc[1];
        if (ccnt <= 1) { /* U-turn toward end */
            j->heading[i] = r | HEAD_TO_END;
            return;
        }
    } else { /* :794-801 */
        cidx = rc[2];
        ccnt = rc[3];
        if (ccnt <= 1) {
            j->heading[i] = r;
            return;
        }
    }
    uint32_t nr;
    if (ccnt == 2) { /* :805-806 */
        nr = conn_at(j, cidx + 1);
    } else { /* :808-811 */
        uint32_t u = rng_next(j->rng_kind, j->rng + 4ull * i);
        uint32_t off = oracle_ranged(u, 1, ccnt);
        nr = conn_at(j, cidx + off);
    }
    const float* np = j->road_pos + 4ull * nr;
    if (np[0] == tx && np[1] == ty) { /* :814-819 */
        j->heading[i] = nr | HEAD_TO_END;
    } else {
        j->heading[i] = nr;
    }
}

static void* step_worker(void* arg) {
    step_job* j = (step_job*)arg;
    for (uint32_t t = 0; t < j->ticks; t++)
        for (uint32_t i = j->begin; i < j->end; i++) step_entity(j, i);
    return NULL;
}

void oracle_step(uint32_t num_roads, const float* road_pos, const uint32_t* road_conn,
                 uint32_t num_conn, const uint32_t* conn, uint32_t n, uint32_t rng_kind, float dt,
                 const float* factor, uint32_t ticks, float* pos, uint32_t* heading, uint32_t* rng,
                 const float* speed, int threads) {
    if (threads <= 0) threads = 1;
    if ((uint32_t)threads > n) threads = n ? (int)n : 1;
    step_job base = {num_roads, road_pos, road_conn, num_conn, conn, rng_kind, dt, factor, ticks,
                     pos, heading, rng, speed, 0, n};
    if (threads == 1) {
        step_worker(&base);
        return;
    }
    /* entities are independent in the move step, so each thread runs all ticks
     * over its own range (the shader_validation driver splits ranges the same
     * way, shader_validation/src/main.cpp:1074-1080) */
    step_job* jobs = (step_job*)malloc(sizeof(step_job) * (size_t)threads);
    pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int t = 0; t < threads; t++) {
        jobs[t] = base;
        jobs[t].begin = (uint32_t)((uint64_t)n * (uint64_t)t / (uint64_t)threads);
        jobs[t].end = (uint32_t)((uint64_t)n * (uint64_t)(t + 1) / (uint64_t)threads);
        pthread_create(&tids[t], NULL, step_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(tids[t], NULL);
    free(jobs);
    free(tids);
}

/* ---- neighbour query ------------------------------------------------------ */

/* random_move.comp:551-562 quad_tree_in_range(v1 = other, v2 = self, R):
 * |dx| <= R, |dy| <= R, then distance(v1, v2) = length(v1 - v2) < R. */
int oracle_in_range(float ax, float ay, float bx, float by, float radius) {
    float dx = fabsf(bx - ax);
    if (dx > radius) return 0;
    float dy = fabsf(by - ay);
    if (dy > radius) return 0;
    float ex = ax - bx;
    float ey = ay - by;
    float ex2 = ex * ex;
    float ey2 = ey * ey;
    return sqrtf(ex2 + ey2) < radius;
}

typedef struct {
    uint32_t n;
    const float* pos;
    float radius;
    uint32_t cap;
    uint32_t* count;
    uint32_t* idx;
    /* uniform grid over the entities' bounding box */
    float minx, miny, inv_cell;
    int64_t gx, gy;
    const uint32_t* cell_start; /* gx*gy + 1 */
    const uint32_t* cell_items; /* entity ids, ascending within a cell */
    uint32_t begin, end;
    uint64_t pairs;
} nbr_job;

static inline int64_t cell_of(float v, float vmin, float inv, int64_t g) {
    double c = floor(((double)v - (double)vmin) * (double)inv);
    if (!(c >= 0.0)) return 0;
    if (c >= (double)g) return g - 1;
    return (int64_t)c;
}

static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return (x > y) - (x < y);
}

static void* nbr_worker(void* arg) {
    nbr_job* j = (nbr_job*)arg;
    uint32_t buf_cap = 256;
    uint32_t* buf = (uint32_t*)malloc(sizeof(uint32_t) * buf_cap);
    uint64_t pairs = 0;
    for (uint32_t i = j->begin; i < j->end; i++) {
        float x = j->pos[2ull * i], y = j->pos[2ull * i + 1];
        /* one extra ring of cells on every side: cells are at least R wide */
        int64_t cx0 = cell_of(x, j->minx, j->inv_cell, j->gx) - 1;
        int64_t cx1 = cell_of(x, j->minx, j->inv_cell, j->gx) + 1;
        int64_t cy0 = cell_of(y, j->miny, j->inv_cell, j->gy) - 1;
        int64_t cy1 = cell_of(y, j->miny, j->inv_cell, j->gy) + 1;
        if (cx0 < 0) cx0 = 0;
        if (cy0 < 0) cy0 = 0;
        if (cx1 >= j->gx) cx1 = j->gx - 1;
        if (cy1 >= j->gy) cy1 = j->gy - 1;
        uint32_t k = 0;
        for (int64_t cy = cy0; cy <= cy1; cy++) {
            for (int64_t cx = cx0; cx <= cx1; cx++) {
                int64_t c = cy * j->gx + cx;
                for (uint32_t q = j->cell_start[c]; q < j->cell_start[c + 1]; q++) {
                    uint32_t o = j->cell_items[q];
                    if (o == i) continue;
                    if (!oracle_in_range(j->pos[2ull * o], j->pos[2ull * o + 1], x, y, j->radius)) continue;
                    if (k == buf_cap) {
                        buf_cap *= 2;
                        buf = (uint32_t*)realloc(buf, sizeof(uint32_t) * buf_cap);
                    }
                    buf[k++] = o;
                    if (o < i) pairs++;
                }
            }
        }
        j->count[i] = k;
        if (j->idx && j->cap) {
            qsort(buf, k, sizeof(uint32_t), cmp_u32);
            uint32_t* out = j->idx + (uint64_t)i * j->cap;
            for (uint32_t q = 0; q < j->cap; q++) out[q] = q < k ? buf[q] : 0xffffffffu;
        }
    }
    free(buf);
    j->pairs = pairs;
    return NULL;
}

uint64_t oracle_neighbours(uint32_t n, const float* pos, float radius, uint32_t cap,
                           uint32_t* count, uint32_t* idx, int threads) {
    if (n == 0) return 0;
    float minx = pos[0], maxx = pos[0], miny = pos[1], maxy = pos[1];
    for (uint32_t i = 1; i < n; i++) {
        float x = pos[2ull * i], y = pos[2ull * i + 1];
        if (x < minx) minx = x;
        if (x > maxx) maxx = x;
        if (y < miny) miny = y;
        if (y > maxy) maxy = y;
    }
    double cell = radius > 0 ? (double)radius : 1.0;
    double w = (double)maxx - (double)minx, h = (double)maxy - (double)miny;
    while ((w / cell + 1.0) * (h / cell + 1.0) > 4.0 * (double)n + 4096.0) cell *= 2.0;
    int64_t gx = (int64_t)(w / cell) + 1, gy = (int64_t)(h / cell) + 1;
    float inv = (float)(1.0 / cell);
    uint32_t* start = (uint32_t*)calloc((size_t)(gx * gy + 1), sizeof(uint32_t));
    uint32_t* items = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* cellid = (uint32_t*)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; i++) {
        int64_t c = cell_of(pos[2ull * i + 1], miny, inv, gy) * gx + cell_of(pos[2ull * i], minx, inv, gx);
        cellid[i] = (uint32_t)c;
        start[c + 1]++;
    }
    for (int64_t c = 0; c < gx * gy; c++) start[c + 1] += start[c];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(gx * gy));
    memcpy(fill, start, sizeof(uint32_t) * (size_t)(gx * gy));
    for (uint32_t i = 0; i < n; i++) items[fill[cellid[i]]++] = i;
    free(fill);
    free(cellid);

    if (threads <= 0) threads = 1;
    if ((uint32_t)threads > n) threads = (int)n;
    nbr_job* jobs = (nbr_job*)malloc(sizeof(nbr_job) * (size_t)threads);
    pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int t = 0; t < threads; t++) {
        nbr_job jb = {n, pos, radius, cap, count, idx, minx, miny, inv, gx, gy, start, items,
                      (uint32_t)((uint64_t)n * (uint64_t)t / (uint64_t)threads),
                      (uint32_t)((uint64_t)n * (uint64_t)(t + 1) / (uint64_t)threads), 0};
        jobs[t] = jb;
        if (threads == 1)
            nbr_worker(&jobs[t]);
        else
            pthread_create(&tids[t], NULL, nbr_worker, &jobs[t]);
    }
    uint64_t pairs = 0;
    for (int t = 0; t < threads; t++) {
        if (threads > 1) pthread_join(tids[t], NULL);
        pairs += jobs[t].pairs;
    }
    free(jobs);
    free(tids);
    free(start);
    free(items);
    return pairs;
}
