// Reference-layout quad tree export for Simulator::get_quad_tree_nodes.
//
// The GPU path indexes entities by sorted tile keys and keeps no tree.  Tools
// that draw the reference's quad-tree grid (QuadTreeGridGlObject.cpp:45-46) get
// the tree the reference would build by inserting the entities one after another
// in id order: node layout GpuQuadTree.hpp:14-41 (64 bytes), entity links
// GpuQuadTree.hpp:44-62 (20 bytes), insertion rules of random_move.comp:309-371
// (descend by the node centre; a leaf splits when it holds node_cap entities,
// unless it is at max_depth or the new entity sits exactly on the leaf's first
// entity; a split moves the leaf's list into four children allocated from the
// lowest free node indices, random_move.comp:175-220, 280-299; lists grow at the
// front, :143-160).  The reference's concurrent GPU build gives different (and
// non-deterministic) node numbering; this sequential build is deterministic.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "msim_internal.h"

namespace msim {

namespace {

constexpr uint32_t kTypeNode = 1, kTypeEntity = 2;

struct Node {  // GpuQuadTree.hpp:14-41
    int32_t acquireLock, writeLock, readerLock;
    float offsetX, offsetY, width, height;
    uint32_t contentType, entityCount, first, prevNodeIndex;
    uint32_t nextTL, nextTR, nextBL, nextBR, padding;
};
static_assert(sizeof(Node) == 64, "node layout");

struct Link {  // GpuQuadTree.hpp:44-62
    uint32_t nodeIndex, typeNext, next, typePrev, prev;
};
static_assert(sizeof(Link) == 20, "entity link layout");

struct Tree {
    Node* nodes;
    uint32_t capacity;
    uint32_t next_free = 1;
    std::vector<Link> links;
    const float* pos;
    uint32_t max_depth, node_cap;
    bool overflow = false;

    void append(uint32_t node, uint32_t e) {  // random_move.comp:143-160
        Node& nd = nodes[node];
        if (nd.entityCount == 0) {
            nd.first = e;
            links[e] = Link{node, 0u, 0u, 0u, 0u};
        } else {
            uint32_t old = nd.first;
            links[e] = Link{node, kTypeEntity, old, 0u, 0u};
            links[old].typePrev = kTypeEntity;
            links[old].prev = e;
            nd.first = e;
        }
        nd.entityCount++;
    }
    uint32_t child_for(const Node& nd, float x, float y) const {
        float cx = nd.offsetX + nd.width / 2.0f;
        float cy = nd.offsetY + nd.height / 2.0f;
        if (x < cx) return y < cy ? nd.nextTL : nd.nextBL;
        return y < cy ? nd.nextTR : nd.nextBR;
    }
    void init_child(uint32_t idx, uint32_t parent, float ox, float oy, float w, float h) {  // :265-278
        Node& c = nodes[idx];
        c.acquireLock = c.writeLock = c.readerLock = 0;
        c.offsetX = ox;
        c.offsetY = oy;
        c.width = w;
        c.height = h;
        c.prevNodeIndex = parent;
        c.contentType = kTypeEntity;
        c.entityCount = 0;
    }
    bool split(uint32_t node) {  // :280-299 with the list move of :222-278
        if (next_free + 4 > capacity) {
            overflow = true;
            return false;
        }
        Node& nd = nodes[node];
        nd.contentType = kTypeNode;
        uint32_t a = next_free++, b = next_free++, c = next_free++, d = next_free++;
        float w = nd.width / 2.0f, h = nd.height / 2.0f;
        nd.nextTL = a;
        init_child(a, node, nd.offsetX, nd.offsetY, w, h);
        nd.nextTR = b;
        init_child(b, node, nd.offsetX + w, nd.offsetY, w, h);
        nd.nextBL = c;
        init_child(c, node, nd.offsetX, nd.offsetY + h, w, h);
        nd.nextBR = d;
        init_child(d, node, nd.offsetX + w, nd.offsetY + h, w, h);
        uint32_t e = nd.first;
        uint32_t count = nd.entityCount;
        nd.first = 0;
        nd.entityCount = 0;
        for (uint32_t k = 0; k < count; k++) {
            uint32_t nxt = links[e].next;
            links[e].next = 0;
            links[e].typeNext = 0;
            append(child_for(nodes[node], pos[2ull * e], pos[2ull * e + 1]), e);
            e = nxt;
        }
        return true;
    }
    void insert(uint32_t e) {  // :309-371 from the root
        float x = pos[2ull * e], y = pos[2ull * e + 1];
        uint32_t node = 0, depth = 1;
        while (true) {
            Node& nd = nodes[node];
            if (nd.contentType == kTypeNode) {
                node = child_for(nd, x, y);
                depth++;
                continue;
            }
            bool same = nd.entityCount > 0 && pos[2ull * nd.first] == x && pos[2ull * nd.first + 1] == y;
            if (nd.entityCount < node_cap || depth >= max_depth || same || !split(node)) {
                append(node, e);
                return;
            }
        }
    }
};

}  // namespace

int build_quad_tree(const float* pos, uint32_t n, float width, float height, uint32_t max_depth, uint32_t node_cap,
                    void* nodes_out, uint32_t node_capacity, void* links_out, uint32_t* nodes_used) {
    if (!nodes_out || (n && !pos)) return fail(MSIM_ERR_INVALID, "NULL argument");
    if (max_depth < 1 || max_depth > 12) return fail(MSIM_ERR_INVALID, "max_depth must be in [1, 12]");
    if (node_cap < 1) return fail(MSIM_ERR_INVALID, "node_cap must be >= 1");
    uint64_t full = 0;
    for (uint32_t d = 0; d < max_depth; d++) full += 1ull << (2 * d);  // GpuQuadTree.cpp:12-18
    if (node_capacity < full)
        return fail(MSIM_ERR_INVALID, "node_capacity must be >= " + std::to_string(full) + " for max_depth " +
                                          std::to_string(max_depth));
    Tree t;
    t.nodes = static_cast<Node*>(nodes_out);
    t.capacity = node_capacity;
    std::memset(t.nodes, 0, sizeof(Node) * (size_t)node_capacity);
    t.links.assign(n, Link{0, 0, 0, 0, 0});
    t.pos = pos;
    t.max_depth = max_depth;
    t.node_cap = node_cap;
    t.nodes[0].width = width;  // GpuQuadTree.cpp:6-10 init_node_zero
    t.nodes[0].height = height;
    t.nodes[0].contentType = kTypeEntity;
    for (uint32_t e = 0; e < n; e++) t.insert(e);
    if (links_out && n) std::memcpy(links_out, t.links.data(), sizeof(Link) * (size_t)n);
    if (nodes_used) *nodes_used = t.next_free;
    return MSIM_OK;
}

}  // namespace msim

extern "C" int msim_quad_tree_build(const float* pos, uint32_t n, float width, float height, uint32_t max_depth,
                                    uint32_t node_cap, void* nodes, uint32_t node_capacity, void* links,
                                    uint32_t* nodes_used) {
    return msim::build_quad_tree(pos, n, width, height, max_depth, node_cap, nodes, node_capacity, links, nodes_used);
}
