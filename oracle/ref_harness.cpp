// Harness around the reference's own CPU quad tree and collision code
// (shader_validation/src/main.cpp of COM8/movement-sim), compiled from the
// reference source where it lies by oracle/build_oracle.py into oracle/_ref.
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle's neighbour predicate against the
// reference's quad tree (insert: main.cpp:309-371, query: main.cpp:~750-919) and
// runs the reference's known-answer test run_collision_detection_test_1
// (main.cpp:1137-1199).  The reference file is included, not copied; its main()
// is renamed so this library has no entry point.
#include <cstring>

#define main msim_reference_shader_validation_main
#include "main.cpp"  // resolved through -I <reference>/shader_validation/src
#undef main

extern "C" {

// Compile-time capacity of the reference's static arrays (main.cpp:151).
int ref_max_entities() { return (int)NUM_ENTITIES; }

static int build_tree(unsigned n, const float* xy, float world_w, float world_h, float radius, unsigned node_cap) {
    if (n > NUM_ENTITIES) return -1;
    reset();
    pushConsts.worldSizeX = world_w;
    pushConsts.worldSizeY = world_h;
    pushConsts.collisionRadius = radius;
    NODE_ENTITY_CAP = node_cap;
    // the tree part of init() (main.cpp:1006-1020) without its random entity moves
    quadTreeNodes[0].width = world_w;
    quadTreeNodes[0].height = world_h;
    quadTreeNodes[0].contentType = TYPE_ENTITY;
    quadTreeNodeUsedStatus[1] = 2;
    for (unsigned i = 0; i < n; i++) {
        entities[i].pos = vec2(xy[2 * i], xy[2 * i + 1]);
        quad_tree_insert(i, 0, 1);
    }
    validate_entity_count(n);
    return 0;
}

// Inserts entities 0..n-1 at xy into an empty reference quad tree over a
// world_w x world_h world (leaf capacity node_cap, depth limit 8), then calls
// quad_tree_check_collisions(i) for each i in order.  events[i] = how often that
// call bumped the collision counter debugData[1] (main.cpp:~743); the traversal
// can visit a pair more than once, so this over-counts.  The distinct partners
// come from the colour writes: quad_tree_collision(i, j) paints both entities
// (main.cpp:~741-742), so after clearing all colours the painted j != i are
// exactly the distinct j < i the reference found.  lower[i] = their number;
// ids (may be NULL) receives them ascending, max_ids per entity.
int ref_lower_sets(unsigned n, const float* xy, float world_w, float world_h, float radius, unsigned node_cap,
                   unsigned* lower, unsigned* events, unsigned* ids, unsigned max_ids) {
    if (build_tree(n, xy, world_w, world_h, radius, node_cap) != 0) return -1;
    for (unsigned i = 0; i < n; i++) {
        for (unsigned j = 0; j < n; j++) entities[j].color = vec4(0);
        unsigned before = debugData[1];
        quad_tree_check_collisions(i);
        events[i] = debugData[1] - before;
        unsigned k = 0;
        for (unsigned j = 0; j < n; j++) {
            if (j == i || entities[j].color.x != 1.0f) continue;
            if (ids && k < max_ids) ids[(size_t)i * max_ids + k] = j;
            k++;
        }
        lower[i] = k;
    }
    return 0;
}

// The reference's tree after inserting entities 0..n-1 in order (single thread):
// nodes_out receives NUM_NODES records of 16 words (GpuQuadTree.hpp:14-41 field
// order), links_out n records of 5 words.
int ref_export_tree(unsigned n, const float* xy, float world_w, float world_h, unsigned node_cap, unsigned* nodes_out,
                    unsigned* links_out) {
    if (build_tree(n, xy, world_w, world_h, 10.0f, node_cap) != 0) return -1;
    for (size_t k = 0; k < NUM_NODES; k++) {
        const QuadTreeNodeDescriptor& q = quadTreeNodes[k];
        unsigned* o = nodes_out + 16 * k;
        int a = q.acquireLock, w = q.writeLock, r = q.readerLock;
        std::memcpy(o + 0, &a, 4);
        std::memcpy(o + 1, &w, 4);
        std::memcpy(o + 2, &r, 4);
        std::memcpy(o + 3, &q.offsetX, 4);
        std::memcpy(o + 4, &q.offsetY, 4);
        std::memcpy(o + 5, &q.width, 4);
        std::memcpy(o + 6, &q.height, 4);
        o[7] = q.contentType;
        o[8] = q.entityCount;
        o[9] = q.first;
        o[10] = q.prevNodeIndex;
        o[11] = q.nextTL;
        o[12] = q.nextTR;
        o[13] = q.nextBL;
        o[14] = q.nextBR;
        o[15] = q.padding;
    }
    for (unsigned i = 0; i < n; i++) {
        const QuadTreeEntityDescriptor& e = quadTreeEntities[i];
        unsigned* o = links_out + 5 * i;
        o[0] = e.nodeIndex;
        o[1] = e.typeNext;
        o[2] = e.next;
        o[3] = e.typePrev;
        o[4] = e.prev;
    }
    return 0;
}

// The reference's known-answer test, with its own world, radius and leaf
// capacity (main.cpp:152-155, 240).  Its asserts abort on failure.
int ref_collision_test_1() {
    pushConsts.worldSizeX = 29007.4609f;
    pushConsts.worldSizeY = 16463.7656f;
    pushConsts.collisionRadius = COLLISION_RADIUS;
    NODE_ENTITY_CAP = 100;
    run_collision_detection_test_1();
    return 0;
}

}  // extern "C"
