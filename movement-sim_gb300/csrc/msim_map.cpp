// Map input/output: the reference JSON map format (loader and writer), the
// synthetic lattice generator and map validation.
//
// Loader semantics follow Map::load_from_file (src/sim/Map.cpp:28-150): required
// fields, numbers converted to float (nlohmann's get_to(float) from the parsed
// number), roads whose start equals their end skipped without renumbering the
// connection list (Map.cpp:124-128).  The writer emits the layout of
// map/generate_map.py:152-160 (Map.to_json) and the generator reproduces the
// connection-list semantics of generate_map.py:234-258.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "msim_internal.h"

namespace msim {

namespace {

// ---- minimal JSON DOM ------------------------------------------------------
struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    bool num_is_uint = false;  // literal was a non-negative integer
    uint64_t num_uint = 0;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;

    const JValue* get(const char* key) const {
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

class JParser {
   public:
    JParser(const char* s, size_t n) : p_(s), end_(s + n) {}

    bool parse(JValue& v, std::string& err) {
        skip_ws();
        if (!value(v, 0)) {
            err = err_.empty() ? "malformed JSON" : err_;
            return false;
        }
        skip_ws();
        if (p_ != end_) {
            err = "trailing characters after JSON value";
            return false;
        }
        return true;
    }

   private:
    const char* p_;
    const char* end_;
    std::string err_;

    void skip_ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) p_++;
    }
    bool lit(const char* w) {
        size_t n = std::strlen(w);
        if ((size_t)(end_ - p_) < n || std::memcmp(p_, w, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool value(JValue& v, int depth) {
        if (depth > 64) {
            err_ = "JSON nesting too deep";
            return false;
        }
        skip_ws();
        if (p_ >= end_) return false;
        char c = *p_;
        if (c == '{') return object(v, depth);
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v.kind = JValue::String;
            return string(v.str);
        }
        if (c == 't') {
            v.kind = JValue::Bool;
            v.b = true;
            return lit("true");
        }
        if (c == 'f') {
            v.kind = JValue::Bool;
            v.b = false;
            return lit("false");
        }
        if (c == 'n') {
            v.kind = JValue::Null;
            return lit("null");
        }
        return number(v);
    }
    bool object(JValue& v, int depth) {
        v.kind = JValue::Object;
        p_++;
        skip_ws();
        if (p_ < end_ && *p_ == '}') {
            p_++;
            return true;
        }
        while (true) {
            skip_ws();
            std::string key;
            if (p_ >= end_ || *p_ != '"' || !string(key)) return false;
            skip_ws();
            if (p_ >= end_ || *p_ != ':') return false;
            p_++;
            v.obj.emplace_back(std::move(key), JValue());
            if (!value(v.obj.back().second, depth + 1)) return false;
            skip_ws();
            if (p_ < end_ && *p_ == ',') {
                p_++;
                continue;
            }
            if (p_ < end_ && *p_ == '}') {
                p_++;
                return true;
            }
            return false;
        }
    }
    bool array(JValue& v, int depth) {
        v.kind = JValue::Array;
        p_++;
        skip_ws();
        if (p_ < end_ && *p_ == ']') {
            p_++;
            return true;
        }
        while (true) {
            v.arr.emplace_back();
            if (!value(v.arr.back(), depth + 1)) return false;
            skip_ws();
            if (p_ < end_ && *p_ == ',') {
                p_++;
                continue;
            }
            if (p_ < end_ && *p_ == ']') {
                p_++;
                return true;
            }
            return false;
        }
    }
    bool string(std::string& out) {
        p_++;  // opening quote
        while (p_ < end_ && *p_ != '"') {
            if (*p_ == '\\') {
                p_++;
                if (p_ >= end_) return false;
                char e = *p_;
                if (e == 'u') {
                    if (end_ - p_ < 5) return false;
                    out.push_back('?');  // names and values used here are ASCII
                    p_ += 5;
                    continue;
                }
                const char* map = "\"\"\\\\//b\bf\fn\nr\rt\t";
                bool ok = false;
                for (int i = 0; map[i]; i += 2)
                    if (map[i] == e) {
                        out.push_back(map[i + 1]);
                        ok = true;
                        break;
                    }
                if (!ok) return false;
                p_++;
                continue;
            }
            out.push_back(*p_++);
        }
        if (p_ >= end_) return false;
        p_++;
        return true;
    }
    bool number(JValue& v) {
        const char* s = p_;
        if (p_ < end_ && (*p_ == '-' || *p_ == '+')) p_++;
        bool integral = true;
        while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' ||
                             *p_ == '-' || *p_ == '+')) {
            if (*p_ == '.' || *p_ == 'e' || *p_ == 'E') integral = false;
            p_++;
        }
        if (p_ == s) return false;
        std::string tok(s, p_);
        char* endp = nullptr;
        errno = 0;
        v.kind = JValue::Number;
        v.num = std::strtod(tok.c_str(), &endp);
        if (endp == tok.c_str() || *endp != '\0') {
            err_ = "bad number '" + tok + "'";
            return false;
        }
        if (integral && tok[0] != '-') {
            errno = 0;
            unsigned long long u = std::strtoull(tok.c_str(), &endp, 10);
            if (errno == 0 && *endp == '\0') {
                v.num_is_uint = true;
                v.num_uint = u;
            }
        }
        return true;
    }
};

// nlohmann get_to(float): integers convert from their integer value, other
// numbers from the parsed double (both round to nearest).
bool as_float(const JValue* v, float& out) {
    if (!v || v->kind != JValue::Number) return false;
    out = v->num_is_uint ? (float)v->num_uint : (float)v->num;
    return true;
}

bool as_uint(const JValue* v, uint32_t& out) {
    if (!v || v->kind != JValue::Number || !v->num_is_uint || v->num_uint > 0xffffffffull) return false;
    out = (uint32_t)v->num_uint;
    return true;
}

}  // namespace

int load_map_json(const char* path, MapData& out) {
    if (!path) return fail(MSIM_ERR_INVALID, "map path is NULL");
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) return fail(MSIM_ERR_IO, std::string("failed to open map '") + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str();
    JValue root;
    std::string err;
    JParser parser(text.data(), text.size());
    if (!parser.parse(root, err)) return fail(MSIM_ERR_INVALID, "failed to parse map: " + err);
    if (root.kind != JValue::Object) return fail(MSIM_ERR_INVALID, "failed to parse map: root is not an object");

    MapData m;
    // Map.cpp:42-52
    if (!as_float(root.get("maxDistLat"), m.width))
        return fail(MSIM_ERR_INVALID, "Failed to parse map. 'maxDistLat' field missing.");
    if (!as_float(root.get("maxDistLong"), m.height))
        return fail(MSIM_ERR_INVALID, "Failed to parse map. 'maxDistLong' field missing.");
    const JValue* roads = root.get("roads");
    if (!roads || roads->kind != JValue::Array)
        return fail(MSIM_ERR_INVALID, "Failed to parse map. 'roads' field missing.");
    // Map.cpp:63-131
    for (const JValue& jr : roads->arr) {
        uint32_t cis, ccs, cie, cce;
        float sx, sy, ex, ey;
        if (jr.kind != JValue::Object) return fail(MSIM_ERR_INVALID, "Failed to parse map. road is not an object.");
        if (!as_uint(jr.get("connIndexStart"), cis))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'connIndexStart' field missing.");
        if (!as_uint(jr.get("connCountStart"), ccs))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'connCountStart' field missing.");
        const JValue* js = jr.get("start");
        if (!js) return fail(MSIM_ERR_INVALID, "Failed to parse map. 'start' field missing.");
        if (!as_float(js->get("distLat"), sx))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'distLat' field missing.");
        if (!as_float(js->get("distLong"), sy))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'distLong' field missing.");
        if (!as_uint(jr.get("connIndexEnd"), cie))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'connIndexEnd' field missing.");
        if (!as_uint(jr.get("connCountEnd"), cce))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'connCountEnd' field missing.");
        const JValue* je = jr.get("end");
        if (!je) return fail(MSIM_ERR_INVALID, "Failed to parse map. 'end' field missing.");
        if (!as_float(je->get("distLat"), ex))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'distLat' field missing.");
        if (!as_float(je->get("distLong"), ey))
            return fail(MSIM_ERR_INVALID, "Failed to parse map. 'distLong' field missing.");
        if (sx == ex && sy == ey) {  // Map.cpp:124-128
            m.skipped_zero_length++;
            continue;
        }
        m.road_pos.insert(m.road_pos.end(), {sx, sy, ex, ey});
        m.road_conn.insert(m.road_conn.end(), {cis, ccs, cie, cce});
    }
    // Map.cpp:133-145
    const JValue* conns = root.get("connectionRoadIndexList");
    if (!conns || conns->kind != JValue::Array)
        return fail(MSIM_ERR_INVALID, "Failed to parse map. 'connectionRoadIndexList' field missing.");
    m.connections.reserve(conns->arr.size());
    for (const JValue& c : conns->arr) {
        uint32_t u;
        if (!as_uint(&c, u)) return fail(MSIM_ERR_INVALID, "Failed to parse map. connection is not an unsigned integer.");
        m.connections.push_back(u);
    }
    out = std::move(m);
    return MSIM_OK;
}

int write_map_json(const msim_map& map, const char* path) {
    if (!path) return fail(MSIM_ERR_INVALID, "map path is NULL");
    if (map.num_roads && (!map.road_pos || !map.road_conn)) return fail(MSIM_ERR_INVALID, "map arrays are NULL");
    if (map.num_connections && !map.connections) return fail(MSIM_ERR_INVALID, "map connections are NULL");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(MSIM_ERR_IO, std::string("failed to open '") + path + "' for writing");
    auto coord = [&](float x, float y) {
        std::fprintf(f, "{\"lat\": 0, \"long\": 0, \"distLat\": %.9g, \"distLong\": %.9g}", (double)x, (double)y);
    };
    std::fprintf(f, "{\"minDistLat\": 0, \"maxDistLat\": %.9g, \"minDistLong\": 0, \"maxDistLong\": %.9g, \"roads\": [",
                 (double)map.width, (double)map.height);
    for (uint32_t r = 0; r < map.num_roads; r++) {
        const float* p = map.road_pos + 4ull * r;
        const uint32_t* c = map.road_conn + 4ull * r;
        std::fprintf(f, r ? ", {\"start\": " : "{\"start\": ");
        coord(p[0], p[1]);
        std::fprintf(f, ", \"end\": ");
        coord(p[2], p[3]);
        std::fprintf(f, ", \"connIndexStart\": %u, \"connCountStart\": %u, \"connIndexEnd\": %u, \"connCountEnd\": %u}",
                     c[0], c[1], c[2], c[3]);
    }
    std::fprintf(f, "], \"connectionRoadIndexList\": [");
    for (uint32_t i = 0; i < map.num_connections; i++) std::fprintf(f, i ? ", %u" : "%u", map.connections[i]);
    std::fprintf(f, "]}\n");
    bool ok = std::ferror(f) == 0;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(MSIM_ERR_IO, std::string("failed to write '") + path + "'");
    return MSIM_OK;
}

int validate_map(const msim_map& map) {
    if (map.num_roads && (!map.road_pos || !map.road_conn)) return fail(MSIM_ERR_INVALID, "map arrays are NULL");
    if (map.num_connections && !map.connections) return fail(MSIM_ERR_INVALID, "map connections are NULL");
    if (map.num_roads == 0) return fail(MSIM_ERR_INVALID, "map has no roads");
    if (map.num_roads > 0x7fffffffu) return fail(MSIM_ERR_INVALID, "too many roads for the heading word");
    if (!(map.width > 0.f) || !(map.height > 0.f) || !std::isfinite(map.width) || !std::isfinite(map.height))
        return fail(MSIM_ERR_INVALID, "map width/height must be positive and finite");
    for (uint32_t r = 0; r < map.num_roads; r++) {
        const float* p = map.road_pos + 4ull * r;
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(p[k])) return fail(MSIM_ERR_INVALID, "road " + std::to_string(r) + " has a non-finite coordinate");
        if (p[0] == p[2] && p[1] == p[3]) return fail(MSIM_ERR_INVALID, "road " + std::to_string(r) + " has zero length");
        const uint32_t* c = map.road_conn + 4ull * r;
        for (int e = 0; e < 2; e++) {
            uint64_t idx = c[2 * e], cnt = c[2 * e + 1];
            if (cnt >= 2 && idx + cnt > map.num_connections)
                return fail(MSIM_ERR_OOB, "road " + std::to_string(r) + (e ? " end" : " start") +
                                              ": connection list [" + std::to_string(idx) + ", +" +
                                              std::to_string(cnt) + "] leaves connectionRoadIndexList (" +
                                              std::to_string(map.num_connections) + " entries + 1 pad)");
        }
    }
    for (uint32_t i = 0; i < map.num_connections; i++)
        if (map.connections[i] >= map.num_roads)
            return fail(MSIM_ERR_OOB, "connectionRoadIndexList[" + std::to_string(i) + "] = " +
                                          std::to_string(map.connections[i]) + " is not a road index (" +
                                          std::to_string(map.num_roads) + " roads)");
    return MSIM_OK;
}

int generate_lattice(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob, MapData& out) {
    if (side < 2 || side > 8192) return fail(MSIM_ERR_INVALID, "lattice side must be in [2, 8192]");
    if (!(spacing > 0.f) || !(jitter >= 0.f) || !(2.f * jitter < spacing))
        return fail(MSIM_ERR_INVALID, "need spacing > 0 and 0 <= 2*jitter < spacing");
    if (!(keep_prob > 0.f) || keep_prob > 1.f) return fail(MSIM_ERR_INVALID, "keep_prob must be in (0, 1]");
    const uint64_t L = side, nn = L * L;
    // Node positions: spacing*(a, b) + 2*jitter*u (u in [0,1)), i.e. a jitter of
    // +-jitter around the lattice point shifted by +jitter so that min >= 0.
    std::vector<float> nx(nn), ny(nn);
    for (uint64_t id = 0; id < nn; id++) {
        uint64_t a = id % L, b = id / L;
        double ux = (double)(uint32_t)(draw(seed, 10, id) >> 40) * 0x1p-24;
        double uy = (double)(uint32_t)(draw(seed, 11, id) >> 40) * 0x1p-24;
        nx[id] = (float)((double)spacing * (double)a + 2.0 * (double)jitter * ux);
        ny[id] = (float)((double)spacing * (double)b + 2.0 * (double)jitter * uy);
    }
    auto keep = [&](uint64_t stream, uint64_t id) {
        return (double)(draw(seed, stream, id) >> 11) * 0x1p-53 < (double)keep_prob;
    };
    std::vector<uint8_t> eh(nn, 0), ev(nn, 0);  // edge to (a+1, b) / (a, b+1)
    for (uint64_t id = 0; id < nn; id++) {
        uint64_t a = id % L, b = id / L;
        if (a + 1 < L) eh[id] = keep(12, id);
        if (b + 1 < L) ev[id] = keep(13, id);
    }
    // largest connected component (union-find; ties -> the one with the smallest node id)
    std::vector<uint32_t> parent(nn);
    std::iota(parent.begin(), parent.end(), 0u);
    auto find = [&](uint32_t x) {
        while (parent[x] != x) {
            parent[x] = parent[parent[x]];
            x = parent[x];
        }
        return x;
    };
    auto unite = [&](uint32_t x, uint32_t y) {
        x = find(x);
        y = find(y);
        if (x != y) parent[std::max(x, y)] = std::min(x, y);
    };
    for (uint64_t id = 0; id < nn; id++) {
        if (eh[id]) unite((uint32_t)id, (uint32_t)(id + 1));
        if (ev[id]) unite((uint32_t)id, (uint32_t)(id + L));
    }
    std::vector<uint32_t> size(nn, 0);
    for (uint64_t id = 0; id < nn; id++) size[find((uint32_t)id)]++;
    uint32_t best = 0;
    for (uint64_t id = 0; id < nn; id++)
        if (size[id] > size[best]) best = (uint32_t)id;
    if (size[best] < 2) return fail(MSIM_ERR_INVALID, "lattice has no edges; raise keep_prob");
    std::vector<uint8_t> in(nn);
    for (uint64_t id = 0; id < nn; id++) in[id] = find((uint32_t)id) == best;

    // roads in node order (horizontal then vertical edge); start = lower node id
    std::vector<uint32_t> rs, re;
    for (uint64_t id = 0; id < nn; id++) {
        if (!in[id]) continue;
        if (eh[id]) {
            rs.push_back((uint32_t)id);
            re.push_back((uint32_t)(id + 1));
        }
        if (ev[id]) {
            rs.push_back((uint32_t)id);
            re.push_back((uint32_t)(id + L));
        }
    }
    const uint32_t R = (uint32_t)rs.size();
    MapData m;
    m.road_pos.resize(4ull * R);
    m.road_conn.assign(4ull * R, 0);
    float maxx = 0.f, maxy = 0.f;
    for (uint32_t r = 0; r < R; r++) {
        m.road_pos[4ull * r + 0] = nx[rs[r]];
        m.road_pos[4ull * r + 1] = ny[rs[r]];
        m.road_pos[4ull * r + 2] = nx[re[r]];
        m.road_pos[4ull * r + 3] = ny[re[r]];
        maxx = std::max(maxx, std::max(nx[rs[r]], nx[re[r]]));
        maxy = std::max(maxy, std::max(ny[rs[r]], ny[re[r]]));
    }
    // incident roads per node, ascending road id (CSR)
    std::vector<uint32_t> deg(nn + 1, 0);
    for (uint32_t r = 0; r < R; r++) {
        deg[rs[r] + 1]++;
        deg[re[r] + 1]++;
    }
    for (uint64_t id = 0; id < nn; id++) deg[id + 1] += deg[id];
    std::vector<uint32_t> inc(deg[nn]);
    std::vector<uint32_t> fillp(deg.begin(), deg.end() - 1);
    for (uint32_t r = 0; r < R; r++) {  // ascending r -> each list ascending
        inc[fillp[rs[r]]++] = r;
        inc[fillp[re[r]]++] = r;
    }
    // generate_map.py:241-258: one list per node; a road whose end is the node is
    // appended twice; count = number of distinct incident roads
    for (uint64_t id = 0; id < nn; id++) {
        uint32_t d = deg[id + 1] - deg[id];
        if (d == 0) continue;
        uint32_t idx = (uint32_t)m.connections.size();
        for (uint32_t k = deg[id]; k < deg[id + 1]; k++) {
            uint32_t r = inc[k];
            m.connections.push_back(r);
            if (rs[r] == id) {
                m.road_conn[4ull * r + 0] = idx;
                m.road_conn[4ull * r + 1] = d;
            } else {
                m.connections.push_back(r);
                m.road_conn[4ull * r + 2] = idx;
                m.road_conn[4ull * r + 3] = d;
            }
        }
    }
    m.width = maxx + jitter;
    m.height = maxy + jitter;
    out = std::move(m);
    return MSIM_OK;
}

}  // namespace msim

// ---- C ABI: map functions ---------------------------------------------------
extern "C" {

int msim_map_load_json(const char* path, msim_map_buf** out) {
    if (!out) return msim::fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    std::unique_ptr<msim_map_buf> buf(new (std::nothrow) msim_map_buf());
    if (!buf) return msim::fail(MSIM_ERR_NOMEM, "out of host memory");
    int rc = msim::load_map_json(path, buf->data);
    if (rc != MSIM_OK) return rc;
    *out = buf.release();
    return MSIM_OK;
}

int msim_map_generate_lattice(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob,
                              msim_map_buf** out) {
    if (!out) return msim::fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    std::unique_ptr<msim_map_buf> buf(new (std::nothrow) msim_map_buf());
    if (!buf) return msim::fail(MSIM_ERR_NOMEM, "out of host memory");
    int rc;
    try {
        rc = msim::generate_lattice(side, seed, spacing, jitter, keep_prob, buf->data);
    } catch (const std::bad_alloc&) {
        return msim::fail(MSIM_ERR_NOMEM, "out of host memory");
    }
    if (rc != MSIM_OK) return rc;
    *out = buf.release();
    return MSIM_OK;
}

int msim_map_view(const msim_map_buf* buf, msim_map* out) {
    if (!buf || !out) return msim::fail(MSIM_ERR_INVALID, "NULL argument");
    const msim::MapData& d = buf->data;
    out->num_roads = (uint32_t)(d.road_pos.size() / 4);
    out->num_connections = (uint32_t)d.connections.size();
    out->road_pos = d.road_pos.data();
    out->road_conn = d.road_conn.data();
    out->connections = d.connections.data();
    out->width = d.width;
    out->height = d.height;
    return MSIM_OK;
}

int msim_map_write_json(const msim_map* map, const char* path) {
    if (!map) return msim::fail(MSIM_ERR_INVALID, "map is NULL");
    return msim::write_map_json(*map, path);
}

int msim_map_validate(const msim_map* map) {
    if (!map) return msim::fail(MSIM_ERR_INVALID, "map is NULL");
    return msim::validate_map(*map);
}

void msim_map_free(msim_map_buf* buf) { delete buf; }

}  // extern "C"
