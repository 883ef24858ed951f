// Host-side code of the library (map loader/writer/validator, lattice generator,
// reference-layout quad tree) driven under AddressSanitizer and
// UndefinedBehaviorSanitizer by tests/test_host_sanitizers.py: well-formed inputs
// round-trip, malformed ones (bad indices, zero-length roads, non-finite numbers,
// truncated and mutated JSON) are rejected with a status and no memory error.
// Prints "ok" and exits 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "msim.h"
#include "msim_internal.h"

namespace msim {
// the C ABI's error text lives in msim_capi.cu, which this host-only driver leaves out
int fail(int code, const std::string&) { return code; }
}  // namespace msim

#define REQUIRE(c)                                                        \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

static std::string read_file(const std::string& p) {
    std::string s;
    FILE* f = std::fopen(p.c_str(), "rb");
    if (!f) return s;
    char buf[65536];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, k);
    std::fclose(f);
    return s;
}

static void write_file(const std::string& p, const std::string& s) {
    FILE* f = std::fopen(p.c_str(), "wb");
    if (!f) return;
    std::fwrite(s.data(), 1, s.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    const std::string json = dir + "/map.json", bad = dir + "/bad.json";
    // lattices of several sizes: validate, write, read back, compare
    const uint32_t sides[] = {2, 3, 8, 33, 100};
    for (uint32_t side : sides) {
        msim_map_buf* b = nullptr;
        REQUIRE(msim_map_generate_lattice(side, 1000 + side, 50.f, 10.f, 0.9f, &b) == MSIM_OK);
        msim_map m{};
        REQUIRE(msim_map_view(b, &m) == MSIM_OK);
        REQUIRE(msim_map_validate(&m) == MSIM_OK);
        REQUIRE(msim_map_write_json(&m, json.c_str()) == MSIM_OK);
        msim_map_buf* b2 = nullptr;
        REQUIRE(msim_map_load_json(json.c_str(), &b2) == MSIM_OK);
        msim_map m2{};
        REQUIRE(msim_map_view(b2, &m2) == MSIM_OK);
        REQUIRE(m2.num_roads == m.num_roads && m2.num_connections == m.num_connections);
        REQUIRE(std::memcmp(m.road_pos, m2.road_pos, 16u * m.num_roads) == 0);
        REQUIRE(std::memcmp(m.road_conn, m2.road_conn, 16u * m.num_roads) == 0);
        REQUIRE(std::memcmp(m.connections, m2.connections, 4u * m.num_connections) == 0);
        msim_map_free(b2);
        // quad tree over points on the map (reference layout, depth 8, leaf cap 10)
        std::mt19937 g(side);
        std::uniform_real_distribution<float> ux(0.f, m.width), uy(0.f, m.height);
        const uint32_t n = 3000;
        std::vector<float> pos(2 * n);
        for (uint32_t i = 0; i < n; i++) {
            pos[2 * i] = ux(g);
            pos[2 * i + 1] = uy(g);
        }
        std::vector<unsigned char> nodes(64u * 21845u), links(20u * n);
        uint32_t used = 0;
        REQUIRE(msim_quad_tree_build(pos.data(), n, m.width, m.height, 8, 10, nodes.data(), 21845, links.data(),
                                     &used) == MSIM_OK);
        REQUIRE(used >= 1 && used <= 21845);
        REQUIRE(msim_quad_tree_build(pos.data(), n, m.width, m.height, 8, 10, nodes.data(), 4, links.data(),
                                     &used) != MSIM_OK);  // too few nodes for the tree
        msim_map_free(b);
    }
    // invalid maps
    {
        float rp[8] = {0, 0, 10, 0, 10, 0, 10, 10};
        uint32_t rc[8] = {0, 0, 0, 2, 0, 2, 0, 0};
        uint32_t cl[2] = {0, 1};
        msim_map m{2, 2, rp, rc, cl, 20.f, 20.f};
        REQUIRE(msim_map_validate(&m) == MSIM_OK);
        cl[1] = 7;  // not a road index
        REQUIRE(msim_map_validate(&m) == MSIM_ERR_OOB);
        cl[1] = 1;
        rc[3] = 5;  // list leaves the connection array
        REQUIRE(msim_map_validate(&m) == MSIM_ERR_OOB);
        rc[3] = 2;
        rp[2] = 0.f;  // zero-length road 0
        REQUIRE(msim_map_validate(&m) == MSIM_ERR_INVALID);
        rp[2] = std::nanf("");
        REQUIRE(msim_map_validate(&m) == MSIM_ERR_INVALID);
        msim_map_buf* b = nullptr;
        REQUIRE(msim_map_generate_lattice(1, 1, 50.f, 10.f, 0.9f, &b) == MSIM_ERR_INVALID && !b);
        REQUIRE(msim_map_generate_lattice(8, 1, 50.f, 30.f, 0.9f, &b) == MSIM_ERR_INVALID && !b);
    }
    // malformed JSON: empty, truncated at every few bytes, and random byte mutations
    {
        msim_map_buf* b = nullptr;
        REQUIRE(msim_map_load_json((dir + "/missing.json").c_str(), &b) != MSIM_OK && !b);
        write_file(bad, "");
        REQUIRE(msim_map_load_json(bad.c_str(), &b) != MSIM_OK && !b);
        msim_map_buf* src = nullptr;
        REQUIRE(msim_map_generate_lattice(4, 7, 50.f, 10.f, 0.9f, &src) == MSIM_OK);
        msim_map m{};
        msim_map_view(src, &m);
        REQUIRE(msim_map_write_json(&m, json.c_str()) == MSIM_OK);
        const std::string good = read_file(json);
        REQUIRE(!good.empty());
        for (size_t cut = 0; cut < good.size(); cut += 13) {
            write_file(bad, good.substr(0, cut));
            if (msim_map_load_json(bad.c_str(), &b) == MSIM_OK) msim_map_free(b);
            b = nullptr;
        }
        std::mt19937 g(42);
        const char pool[] = "{}[]:,\"-+.eE0123456789 \ntrufalsn\\x";
        for (int t = 0; t < 400; t++) {
            std::string s = good;
            const int edits = 1 + (int)(g() % 4);
            for (int e = 0; e < edits; e++) s[g() % s.size()] = pool[g() % (sizeof(pool) - 1)];
            write_file(bad, s);
            if (msim_map_load_json(bad.c_str(), &b) == MSIM_OK) {
                msim_map mm{};
                msim_map_view(b, &mm);
                msim_map_validate(&mm);  // any status; no memory error
                msim_map_free(b);
            }
            b = nullptr;
        }
        msim_map_free(src);
    }
    std::printf("ok\n");
    return 0;
}
