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

/* ---- synthetic lattice road map ------------------------------------------------ */

/* The synthetic L x L intersection lattice of the workloads, restated here so that
 * the CPU legs need nothing of the product: node (a, b) at spacing*(a, b) plus a
 * uniform offset in [0, 2*jitter) per axis (draw streams 10 and 11), the edge to
 * (a+1, b) kept when draw stream 12 < keep_prob and the edge to (a, b+1) when
 * stream 13 < keep_prob, the largest connected component kept (ties: the one
 * holding the smallest node id).  Roads are numbered in node order, the edge to
 * (a+1, b) before the edge to (a, b+1), and start at their lower node.  The
 * connection lists follow map/generate_map.py:234-258: one list per node, every
 * incident road once in ascending road id, a road that ENDS at the node appended a
 * second time, and count = the number of distinct incident roads.  World size =
 * largest endpoint coordinate + jitter (Map.cpp:42-52 maxDistLat/maxDistLong). */
struct oracle_lattice {
    uint32_t num_roads, num_conn;
    float width, height;
    float* road_pos;     /* 4 per road */
    uint32_t* road_conn; /* 4 per road */
    uint32_t* conn;
};

static int lattice_kept(uint64_t seed, uint64_t stream, uint64_t id, float keep_prob) {
    return (double)(oracle_draw(seed, stream, id) >> 11) * 0x1p-53 < (double)keep_prob;
}

void oracle_lattice_free(oracle_lattice* m) {
    if (!m) return;
    free(m->road_pos);
    free(m->road_conn);
    free(m->conn);
    free(m);
}

oracle_lattice* oracle_lattice_new(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob) {
    if (side < 2 || side > 8192 || !(spacing > 0.f) || !(jitter >= 0.f) || !(2.f * jitter < spacing) ||
        !(keep_prob > 0.f) || keep_prob > 1.f)
        return NULL;
    const uint64_t L = side, nn = L * L;
    float* nx = (float*)malloc(sizeof(float) * nn);
    float* ny = (float*)malloc(sizeof(float) * nn);
    uint8_t* edge = (uint8_t*)calloc(nn, 1); /* bit 0: to (a+1, b), bit 1: to (a, b+1) */
    int32_t* label = (int32_t*)malloc(sizeof(int32_t) * nn);
    uint32_t* queue = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    int64_t* road_h = (int64_t*)malloc(sizeof(int64_t) * nn);
    int64_t* road_v = (int64_t*)malloc(sizeof(int64_t) * nn);
    oracle_lattice* m = (oracle_lattice*)calloc(1, sizeof(oracle_lattice));
    if (!nx || !ny || !edge || !label || !queue || !road_h || !road_v || !m) goto fail;
    for (uint64_t id = 0; id < nn; id++) {
        uint64_t a = id % L, b = id / L;
        double ux = (double)(uint32_t)(oracle_draw(seed, 10, id) >> 40) * 0x1p-24;
        double uy = (double)(uint32_t)(oracle_draw(seed, 11, id) >> 40) * 0x1p-24;
        nx[id] = (float)((double)spacing * (double)a + 2.0 * (double)jitter * ux);
        ny[id] = (float)((double)spacing * (double)b + 2.0 * (double)jitter * uy);
        if (a + 1 < L && lattice_kept(seed, 12, id, keep_prob)) edge[id] |= 1;
        if (b + 1 < L && lattice_kept(seed, 13, id, keep_prob)) edge[id] |= 2;
    }
    /* components by breadth-first search from the smallest unlabelled node: each
     * component's first node is its smallest id, so the first largest one wins ties */
    for (uint64_t id = 0; id < nn; id++) label[id] = -1;
    int32_t best = -1, labels = 0;
    uint64_t best_size = 0;
    for (uint64_t s0 = 0; s0 < nn; s0++) {
        if (label[s0] >= 0) continue;
        uint64_t head = 0, tail = 0;
        label[s0] = labels;
        queue[tail++] = (uint32_t)s0;
        while (head < tail) {
            uint64_t v = queue[head++];
            uint64_t a = v % L, b = v / L;
            uint64_t nb[4];
            int k = 0;
            if (edge[v] & 1) nb[k++] = v + 1;
            if (edge[v] & 2) nb[k++] = v + L;
            if (a > 0 && (edge[v - 1] & 1)) nb[k++] = v - 1;
            if (b > 0 && (edge[v - L] & 2)) nb[k++] = v - L;
            for (int q = 0; q < k; q++)
                if (label[nb[q]] < 0) {
                    label[nb[q]] = labels;
                    queue[tail++] = (uint32_t)nb[q];
                }
        }
        if (tail > best_size) {
            best_size = tail;
            best = labels;
        }
        labels++;
    }
    if (best_size < 2) goto fail;
    /* roads in node order */
    uint64_t R = 0;
    for (uint64_t id = 0; id < nn; id++) {
        road_h[id] = road_v[id] = -1;
        if (label[id] != best) continue;
        if (edge[id] & 1) road_h[id] = (int64_t)R++;
        if (edge[id] & 2) road_v[id] = (int64_t)R++;
    }
    m->num_roads = (uint32_t)R;
    m->road_pos = (float*)malloc(sizeof(float) * 4 * R);
    m->road_conn = (uint32_t*)calloc(4 * R, sizeof(uint32_t));
    m->conn = (uint32_t*)malloc(sizeof(uint32_t) * 6 * R); /* <= 2 entries per road end */
    if (!m->road_pos || !m->road_conn || !m->conn) goto fail;
    float maxx = 0.f, maxy = 0.f;
    for (uint64_t id = 0; id < nn; id++) {
        for (int dir = 0; dir < 2; dir++) {
            int64_t r = dir ? road_v[id] : road_h[id];
            if (r < 0) continue;
            uint64_t e = dir ? id + L : id + 1;
            float* p = m->road_pos + 4 * r;
            p[0] = nx[id];
            p[1] = ny[id];
            p[2] = nx[e];
            p[3] = ny[e];
            if (p[0] > maxx) maxx = p[0];
            if (p[2] > maxx) maxx = p[2];
            if (p[1] > maxy) maxy = p[1];
            if (p[3] > maxy) maxy = p[3];
        }
    }
    /* one connection list per node; incident roads ascending */
    uint64_t C = 0;
    for (uint64_t v = 0; v < nn; v++) {
        uint64_t a = v % L, b = v / L;
        int64_t inc[4];
        int ends[4];
        int d = 0;
        if (b > 0 && road_v[v - L] >= 0) { inc[d] = road_v[v - L]; ends[d++] = 1; }
        if (a > 0 && road_h[v - 1] >= 0) { inc[d] = road_h[v - 1]; ends[d++] = 1; }
        if (road_h[v] >= 0) { inc[d] = road_h[v]; ends[d++] = 0; }
        if (road_v[v] >= 0) { inc[d] = road_v[v]; ends[d++] = 0; }
        if (d == 0) continue;
        for (int i = 1; i < d; i++) /* insertion sort by road id */
            for (int j = i; j > 0 && inc[j - 1] > inc[j]; j--) {
                int64_t t = inc[j]; inc[j] = inc[j - 1]; inc[j - 1] = t;
                int te = ends[j]; ends[j] = ends[j - 1]; ends[j - 1] = te;
            }
        uint32_t first = (uint32_t)C;
        for (int q = 0; q < d; q++) {
            uint32_t r = (uint32_t)inc[q];
            m->conn[C++] = r;
            if (ends[q]) {
                m->conn[C++] = r;
                m->road_conn[4ull * r + 2] = first;
                m->road_conn[4ull * r + 3] = (uint32_t)d;
            } else {
                m->road_conn[4ull * r + 0] = first;
                m->road_conn[4ull * r + 1] = (uint32_t)d;
            }
        }
    }
    m->num_conn = (uint32_t)C;
    m->width = maxx + jitter;
    m->height = maxy + jitter;
    free(nx); free(ny); free(edge); free(label); free(queue); free(road_h); free(road_v);
    return m;
fail:
    free(nx); free(ny); free(edge); free(label); free(queue); free(road_h); free(road_v);
    oracle_lattice_free(m);
    return NULL;
}

void oracle_lattice_info(const oracle_lattice* m, uint32_t* num_roads, uint32_t* num_conn, float* width,
                         float* height) {
    *num_roads = m->num_roads;
    *num_conn = m->num_conn;
    *width = m->width;
    *height = m->height;
}

void oracle_lattice_copy(const oracle_lattice* m, float* road_pos, uint32_t* road_conn, uint32_t* conn) {
    memcpy(road_pos, m->road_pos, sizeof(float) * 4ull * m->num_roads);
    memcpy(road_conn, m->road_conn, sizeof(uint32_t) * 4ull * m->num_roads);
    memcpy(conn, m->conn, sizeof(uint32_t) * m->num_conn);
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
 * SPEED (:750) becomes step = (speed * factor[road]) * dt; 1.4 * 1 * 1 = SPEED.
 * Returns 1 when the entity snapped to its target this tick. */
static int step_entity(const step_job* j, uint32_t i) {
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
        return 0;
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
            return 1;
        }
    } else { /* :794-801 */
        cidx = rc[2];
        ccnt = rc[3];
        if (ccnt <= 1) {
            j->heading[i] = r;
            return 1;
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
    return 1;
}

static void* step_worker(void* arg) {
    step_job* j = (step_job*)arg;
    for (uint32_t t = 0; t < j->ticks; t++)
        for (uint32_t i = j->begin; i < j->end; i++) (void)step_entity(j, i);
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

/* ---- density calibration: FP64 adjoint reference ----------------------------- */

typedef struct {
    step_job sj;               /* map, FP32 state copies, params */
    const float* pos0;
    const uint32_t* head0;
    const uint32_t* rng0;
    double world_w, world_h;
    uint32_t gw, gh;
    const double* lambda;      /* phase 2: dL/dD per cell */
    double* density;           /* phase 1: per-thread accumulator (gw*gh) */
    double* grad_speed;        /* phase 2: per entity */
    double* grad_factor;       /* phase 2: per-thread accumulator (num_roads) */
    int phase;
    int fp64_model;
    uint32_t* sched;           /* phase 1: event bits, sched_words per entity (may be NULL) */
    uint32_t sched_words;
    int fbits;                 /* fraction bits of the fixed-point cell coordinates */
} adj_job;

/* Cell coordinates of position (x, y): u = x * gw / W - 1/2 (cell-centred), the
 * lower cell index and the fraction.  For the FP32 trajectory they are computed
 * as the forward kernel does, in binary32 with the scale rounded to binary32; for
 * the smooth FP64 model in binary64.  *sx, *sy = du/dx, dv/dy. */
static void cell_coords(const adj_job* a, double x, double y, long* i0, long* j0, double* fx, double* fy, double* sx,
                        double* sy) {
    if (a->fp64_model) {
        *sx = (double)a->gw / a->world_w;
        *sy = (double)a->gh / a->world_h;
        const double u = x * *sx - 0.5, v = y * *sy - 0.5;
        const double fi = floor(u), fj = floor(v);
        *i0 = (long)fi;
        *j0 = (long)fj;
        *fx = u - fi;
        *fy = v - fj;
    } else {
        /* binary32 u, then fixed point with fbits fraction bits (truncated) */
        const float isx = (float)((double)a->gw / a->world_w), isy = (float)((double)a->gh / a->world_h);
        const float u = (float)x * isx - 0.5f, v = (float)y * isy - 0.5f;
        const double scale = ldexp(1.0, a->fbits), lim = ldexp(1.0, 30 - a->fbits);
        const double U = floor(fmin(fmax((double)u, -lim), lim) * scale);
        const double V = floor(fmin(fmax((double)v, -lim), lim) * scale);
        const double fi = floor(U / scale), fj = floor(V / scale);
        *sx = (double)isx;
        *sy = (double)isy;
        *i0 = (long)fi;
        *j0 = (long)fj;
        *fx = (U - fi * scale) / scale;
        *fy = (V - fj * scale) / scale;
    }
}

/* Bilinear, cell-centred weights of position (x, y) on the gw x gh grid over
 * [0, W) x [0, H); corners outside the grid are dropped. */
static void splat64(const adj_job* a, double x, double y, double w, double* grid) {
    long i0, j0;
    double fx, fy, sx, sy;
    cell_coords(a, x, y, &i0, &j0, &fx, &fy, &sx, &sy);
    double wt[4] = {(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy};
    long ci[4] = {i0, i0 + 1, i0, i0 + 1}, cj[4] = {j0, j0, j0 + 1, j0 + 1};
    for (int k = 0; k < 4; k++)
        if (ci[k] >= 0 && ci[k] < (long)a->gw && cj[k] >= 0 && cj[k] < (long)a->gh)
            grid[(size_t)cj[k] * a->gw + (size_t)ci[k]] += w * wt[k];
}

static double lam_at(const adj_job* a, long i, long j) {
    if (i < 0 || j < 0 || i >= (long)a->gw || j >= (long)a->gh) return 0.0;
    return a->lambda[(size_t)j * a->gw + (size_t)i];
}

/* d/dp of sum_g lambda_g w_g(p) */
static void splat64_grad(const adj_job* a, double x, double y, double* gx, double* gy) {
    long i0, j0;
    double fx, fy, sx, sy;
    cell_coords(a, x, y, &i0, &j0, &fx, &fy, &sx, &sy);
    double l00 = lam_at(a, i0, j0), l10 = lam_at(a, i0 + 1, j0), l01 = lam_at(a, i0, j0 + 1),
           l11 = lam_at(a, i0 + 1, j0 + 1);
    *gx = ((1 - fy) * (l10 - l00) + fy * (l11 - l01)) * sx;
    *gy = ((1 - fx) * (l01 - l00) + fx * (l11 - l10)) * sy;
}

static void* adj_worker(void* arg) {
    adj_job* a = (adj_job*)arg;
    step_job* j = &a->sj;
    const uint32_t T = j->ticks;
    double* hx = NULL;
    double* hy = NULL;
    uint32_t* hh = NULL;
    unsigned char* hs = NULL;
    if (a->phase == 2) {
        hx = (double*)malloc(sizeof(double) * (T + 1));
        hy = (double*)malloc(sizeof(double) * (T + 1));
        hh = (uint32_t*)malloc(sizeof(uint32_t) * (T + 1));
        hs = (unsigned char*)malloc(T + 1);
    }
    for (uint32_t i = j->begin; i < j->end; i++) {
        j->pos[2ull * i] = a->pos0[2ull * i];
        j->pos[2ull * i + 1] = a->pos0[2ull * i + 1];
        j->heading[i] = a->head0[i];
        memcpy(j->rng + 4ull * i, a->rng0 + 4ull * i, 16);
        double x = a->pos0[2ull * i], y = a->pos0[2ull * i + 1];
        const double s = (double)j->speed[i];
        if (hx) {
            hx[0] = x;
            hy[0] = y;
        }
        for (uint32_t t = 1; t <= T; t++) {
            const uint32_t h = j->heading[i];
            /* the FP32 step: the event schedule, and the trajectory unless fp64_model */
            const int snapped = step_entity(j, i);
            if (!a->fp64_model) {
                x = (double)j->pos[2ull * i];
                y = (double)j->pos[2ull * i + 1];
            } else {
                const uint32_t r = h & HEAD_ROAD;
                const float* rp = j->road_pos + 4ull * r;
                const double tx = (h >> 31) ? rp[2] : rp[0], ty = (h >> 31) ? rp[3] : rp[1];
                if (snapped) {
                    x = tx;
                    y = ty;
                } else {
                    const double l = s * (j->factor ? (double)j->factor[r] : 1.0) * (double)j->dt;
                    const double dx = tx - x, dy = ty - y, L = sqrt(dx * dx + dy * dy);
                    if (L > 0) {
                        x += dx / L * l;
                        y += dy / L * l;
                    }
                }
            }
            if (a->phase == 1) {
                if (a->sched && snapped) a->sched[(size_t)i * a->sched_words + ((t - 1) >> 5)] |= 1u << ((t - 1) & 31u);
                splat64(a, x, y, 1.0 / (double)T, a->density);
            } else {
                hx[t] = x;
                hy[t] = y;
                hh[t] = h;
                hs[t] = (unsigned char)snapped;
            }
        }
        if (a->phase == 2) { /* reverse sweep */
            double ax = 0, ay = 0, gs = 0;
            for (uint32_t t = T; t >= 1; t--) {
                double gx, gy;
                splat64_grad(a, hx[t], hy[t], &gx, &gy);
                ax += gx / (double)T;
                ay += gy / (double)T;
                if (hs[t]) {
                    ax = 0;
                    ay = 0;
                    continue;
                }
                uint32_t r = hh[t] & HEAD_ROAD;
                const float* rp = j->road_pos + 4ull * r;
                double tx = (hh[t] >> 31) ? rp[2] : rp[0], ty = (hh[t] >> 31) ? rp[3] : rp[1];
                double dx = tx - hx[t - 1], dy = ty - hy[t - 1], L = sqrt(dx * dx + dy * dy);
                if (!(L > 0)) continue;
                double f = j->factor ? (double)j->factor[r] : 1.0;
                double l = s * f * (double)j->dt;
                double nx = dx / L, ny = dy / L;
                double gl = nx * ax + ny * ay;
                gs += gl * f * (double)j->dt;
                a->grad_factor[r] += gl * s * (double)j->dt;
                double k = l / L;
                ax -= k * (ax - nx * gl);
                ay -= k * (ay - ny * gl);
            }
            a->grad_speed[i] = gs;
        }
    }
    free(hx);
    free(hy);
    free(hh);
    free(hs);
    return NULL;
}

double oracle_density_adjoint(uint32_t num_roads, const float* road_pos, const uint32_t* road_conn,
                              uint32_t num_conn, const uint32_t* conn, uint32_t n, uint32_t rng_kind, float dt,
                              uint32_t ticks, const float* pos0, const uint32_t* head0, const uint32_t* rng0,
                              const float* speed, const float* factor, float world_w, float world_h, uint32_t gw,
                              uint32_t gh, const float* target, double* density, double* grad_speed,
                              double* grad_factor, int fp64_model, uint32_t* sched, int threads) {
    if (threads <= 0) threads = 1;
    if ((uint32_t)threads > n) threads = n ? (int)n : 1;
    const size_t G = (size_t)gw * gh;
    float* pos = (float*)malloc(sizeof(float) * 2 * (size_t)n + 8);
    uint32_t* head = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n + 4);
    uint32_t* rng = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)n + 16);
    double* dens = (double*)calloc(G * (size_t)threads, sizeof(double));
    double* gf = (double*)calloc((size_t)num_roads * (size_t)threads, sizeof(double));
    double* lambda = (double*)malloc(sizeof(double) * G);
    if (sched) memset(sched, 0, sizeof(uint32_t) * (size_t)n * ((ticks + 31u) / 32u));
    /* largest fraction bits (16..22) with |u| * 2^fbits below 2^30 on this grid */
    int gbits = 0;
    while ((1ull << gbits) < (uint64_t)(gw > gh ? gw : gh) + 1u) gbits++;
    int fbits = 30 - gbits;
    fbits = fbits > 22 ? 22 : (fbits < 16 ? 16 : fbits);
    adj_job* jobs = (adj_job*)malloc(sizeof(adj_job) * (size_t)threads);
    pthread_t* tids = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int phase = 1; phase <= 2; phase++) {
        for (int t = 0; t < threads; t++) {
            step_job sj = {num_roads, road_pos, road_conn, num_conn, conn, rng_kind, dt, factor, ticks, pos, head, rng,
                           speed, (uint32_t)((uint64_t)n * (uint64_t)t / (uint64_t)threads),
                           (uint32_t)((uint64_t)n * (uint64_t)(t + 1) / (uint64_t)threads)};
            adj_job aj = {sj, pos0, head0, rng0, (double)world_w, (double)world_h, gw, gh, lambda,
                          dens + G * (size_t)t, grad_speed, gf + (size_t)num_roads * (size_t)t, phase,
                          fp64_model, sched, (ticks + 31u) / 32u, fbits};
            jobs[t] = aj;
            pthread_create(&tids[t], NULL, adj_worker, &jobs[t]);
        }
        for (int t = 0; t < threads; t++) pthread_join(tids[t], NULL);
        if (phase == 1) { /* D, loss, lambda = dL/dD (thread partials summed in order) */
            for (int t = 1; t < threads; t++)
                for (size_t g = 0; g < G; g++) dens[g] += dens[G * (size_t)t + g];
            for (size_t g = 0; g < G; g++) {
                if (density) density[g] = dens[g];
                lambda[g] = 2.0 / (double)G * (dens[g] - (double)target[g]);
            }
        }
    }
    double loss = 0;
    for (size_t g = 0; g < G; g++) {
        double d = dens[g] - (double)target[g];
        loss += d * d;
    }
    loss /= (double)G;
    for (uint32_t r = 0; r < num_roads; r++) {
        double acc = 0;
        for (int t = 0; t < threads; t++) acc += gf[(size_t)num_roads * (size_t)t + r];
        grad_factor[r] = acc;
    }
    free(pos);
    free(head);
    free(rng);
    free(dens);
    free(gf);
    free(lambda);
    free(jobs);
    free(tids);
    return loss;
}
