/*
 * ref_fmm_driver.cpp -- runs the reference's own FMM kernels on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  The kernel bodies are the reference files
 * src/moment.cl, src/interaction.cl, src/field.cl and src/force.cl, included
 * unmodified through cl_kernel_shim.h (compiled from where they lie by
 * oracle/Makefile; nothing is copied).  This file is the host side: it
 * restates the orchestration of src/open_cl_simulation.cpp:126-616 with the
 * bugs listed below fixed, so that the kernels compute the reference's
 * intended order-0 FMM:
 *   - the octree (absent glade library) is supplied by the caller in
 *     breadth-first form and converted to the reference node_t layout in
 *     pre-order with all eight children materialised (empty ones have
 *     leaf_count 0, which src/interaction.cl:55-56 drops);
 *   - M2M (src/moment.cl:72-160) never runs in the reference
 *     (src/open_cl_simulation.cpp:156-157 resets the loop bound); the
 *     intended sum of child charges is done here on the host;
 *   - interaction slot indices (src/interaction.cl:104-123 discards them)
 *     are assigned here exactly as the kernel intends (per-node counters in
 *     list order);
 *   - everything runs as one batch (no device-size batching, so every
 *     interaction contributes to the integrated forces);
 *   - the node-field kernel's leaf partition (src/field.cl:196-201) is
 *     launched with a local size >= every target's leaf_count, and the leaf
 *     kernel (fixed 8x8 groups, src/field.cl:85-98) is only used when every
 *     leaf holds <= 8 particles (the reference's capacity), where its
 *     partition covers every pair.
 */
#include "cl_kernel_shim.h"

#include "moment.cl"
#include "interaction.cl"
#include "field.cl"
#include "force.cl"

#include <cstring>
#include <vector>

nbody_shim_item nbody_shim_cur;

template <typename F>
static void launch1(size_t gsize, size_t local, F&& f) {
    for (size_t g = 0; g < gsize / local; ++g)
        for (size_t l = 0; l < local; ++l) {
            nbody_shim_cur = nbody_shim_item{{g * local + l, 0, 0}, {l, 0, 0}, {g, 0, 0}, {local, 1, 1}};
            f();
        }
}
template <typename F>
static void launch2(size_t g0, size_t g1, size_t l0, size_t l1, F&& f) {
    for (size_t a = 0; a < g0 / l0; ++a)
        for (size_t b = 0; b < g1 / l1; ++b)
            for (size_t y = 0; y < l1; ++y)
                for (size_t x = 0; x < l0; ++x) {
                    nbody_shim_cur = nbody_shim_item{{a * l0 + x, b * l1 + y, 0}, {x, y, 0}, {a, b, 0}, {l0, l1, 1}};
                    f();
                }
}

struct Tree {
    std::vector<node_t> nodes;
    std::vector<int> pre_of_bfs, bfs_of_pre;
};

/* bfs rows: level, ix, iy, iz, begin, count, parent, child_begin, nchild */
static int convert(Tree& T, const int32_t* bfs, int nbfs, const double* box, int bfs_k, int octant, int parent_pre,
                   int lev, long ix, long iy, long iz, int begin_hint) {
    int idx = (int)T.nodes.size();
    T.nodes.push_back(node_t());
    T.bfs_of_pre.push_back(bfs_k);
    node_t nd;
    std::memset(&nd, 0, sizeof(nd));
    double w = box[3] / (double)(1L << lev);
    nd.position = float4((float)(box[0] + ix * w), (float)(box[1] + iy * w), (float)(box[2] + iz * w), 0.0f);
    nd.dimensions = float4((float)w, (float)w, (float)w, 0.0f);
    nd.depth = (uint)lev;
    nd.parent_index = parent_pre < 0 ? 0 : parent_pre - idx;
    nd.sibling_index = (uint)octant;
    if (bfs_k >= 0) {
        const int32_t* r = bfs + 9 * bfs_k;
        T.pre_of_bfs[bfs_k] = idx;
        nd.leaf_index = (uint)r[4];
        nd.leaf_count = (uint)r[5];
        nd.has_children = r[8] > 0;
        T.nodes[idx] = nd;
        if (r[8] > 0) {
            int next_child = 0;
            for (int d = 0; d < 8; ++d) {
                int ck = -1;
                if (next_child < r[8]) {
                    const int32_t* cr = bfs + 9 * (r[7] + next_child);
                    int cd = (cr[1] & 1) | ((cr[2] & 1) << 1) | ((cr[3] & 1) << 2);
                    if (cd == d) { ck = r[7] + next_child; ++next_child; }
                }
                int cidx = convert(T, bfs, nbfs, box, ck, d, idx, lev + 1, 2 * ix + (d & 1), 2 * iy + ((d >> 1) & 1),
                                   2 * iz + (d >> 2), ck >= 0 ? bfs[9 * ck + 4] : r[4]);
                T.nodes[idx].child_indices[d] = (uint)(cidx - idx);
            }
        }
    } else {
        nd.leaf_index = (uint)begin_hint;
        nd.leaf_count = 0;
        nd.has_children = 0;
        T.nodes[idx] = nd;
    }
    /* offset to the next sibling = subtree size (only read by the M2M kernel) */
    T.nodes[idx].child_indices[8] = (uint)(T.nodes.size() - idx);
    return idx;
}

extern "C" int ref_fmm_run(int n, const float* pos3, const float* vel3, const float* mass, const float* charge,
                           int nbfs, const int32_t* bfs, const double* box, float dt,
                           int pair_cap, int* n_leaf_pairs, int32_t* leaf_pairs, int* n_node_pairs,
                           int32_t* node_pairs, float* f_leaf, float* f_node, float* pos_out, float* vel_out) {
    if (n <= 0 || nbfs <= 0) return -1;
    Tree T;
    T.pre_of_bfs.assign(nbfs, -1);
    convert(T, bfs, nbfs, box, 0, 0, -1, 0, 0, 0, 0, 0);
    std::vector<node_t>& nodes = T.nodes;
    const size_t nn = nodes.size();

    std::vector<leaf_t> leafs(n);
    for (int i = 0; i < n; ++i) {
        std::memset(&leafs[i], 0, sizeof(leaf_t));
        leafs[i].position = float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.0f);
        leafs[i].value.velocity = float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0f);
        leafs[i].value.mass = mass[i];
        leafs[i].value.moment.charge = charge[i];
    }

    /* P2M at childless nodes: src/moment.cl:6-67 (local size 64 as a preferred multiple) */
    std::vector<uint> processed(nn + 64, 0);
    {
        size_t local = 64, groups = nn / local + (nn % local != 0) + (nn == 0);
        launch1(groups * local, local, [&] {
            compute_moments_from_leafs((uint)n, leafs.data(), (uint)nn, nodes.data(), processed.data());
        });
    }
    /* intended M2M of the monopole, deepest node first (children follow parents in pre-order) */
    for (size_t k = nn; k-- > 0;) {
        if (!nodes[k].has_children) continue;
        float s = 0.0f;
        for (int d = 0; d < 8; ++d) s += nodes[k + nodes[k].child_indices[d]].value.moment.charge;
        nodes[k].value.moment.charge = s;
    }

    /* interaction finding: src/open_cl_simulation.cpp:176-268, one batch per tree level */
    std::vector<interaction_t> pending(1);
    std::memset(&pending[0], 0, sizeof(interaction_t));
    pending[0].can_reduce = 1;
    std::vector<interaction_t> leafI, nodeI;
    while (!pending.empty()) {
        std::vector<interaction_t> out(64 * pending.size());
        std::memset(out.data(), 0, sizeof(interaction_t) * out.size());
        launch2(8 * pending.size(), 8, 8, 8, [&] {
            find_interactions((uint)nn, nodes.data(), (uint)pending.size(), pending.data(), out.data());
        });
        pending.clear();
        for (const interaction_t& it : out) {
            if (it.node_a_index == 0 && it.node_b_index == 0) continue;
            if (it.can_reduce) pending.push_back(it);
            else if (!it.can_approx) leafI.push_back(it);
            else nodeI.push_back(it);
        }
    }
    if ((int)leafI.size() > pair_cap || (int)nodeI.size() > pair_cap) return -2;

    /* slot indices as src/interaction.cl:104-123 intends */
    std::vector<uint> numLeafInt(nn, 0), numNodeInt(nn, 0), maxLeafCount(nn, 0);
    for (interaction_t& it : leafI) {
        it.node_a_interaction_index = numLeafInt[it.node_a_index]++;
        it.node_b_interaction_index = numLeafInt[it.node_b_index]++;
    }
    for (interaction_t& it : nodeI) {
        it.node_a_interaction_index = numNodeInt[it.node_a_index]++;
        it.node_b_interaction_index = numNodeInt[it.node_b_index]++;
    }
    {
        size_t m = leafI.size(), local = 64, groups = m / local + (m % local != 0) + (m == 0);
        launch1(groups * local, local, [&] {
            compute_node_max_interactions_leaf_count((uint)nn, nodes.data(), maxLeafCount.data(), (uint)m, leafI.data());
        });
    }
    for (const interaction_t& it : leafI) {
        if (nodes[it.node_a_index].leaf_count > 8 || nodes[it.node_b_index].leaf_count > 8) return -3;
    }

    /* field slot layout: src/open_cl_simulation.cpp:371-484 */
    std::vector<uint> leafFieldIdx(n + 1, 0), nodeFieldIdx(n + 1, 0), nodeParentInt(nn, 0);
    for (size_t k = 0; k < nn; ++k) {
        if (nodes[k].has_children) continue;
        uint nf = maxLeafCount[k] * numLeafInt[k];
        for (uint l = nodes[k].leaf_index; l < nodes[k].leaf_index + nodes[k].leaf_count; ++l)
            leafFieldIdx[l + 1] = leafFieldIdx[l] + nf;
    }
    for (size_t k = 0; k < nn; ++k) {
        if (!nodes[k].has_children) continue;
        for (int d = 0; d < 8; ++d) nodeParentInt[k + nodes[k].child_indices[d]] += numNodeInt[k] + nodeParentInt[k];
    }
    for (size_t k = 0; k < nn; ++k) {
        if (nodes[k].has_children) continue;
        uint nf = numNodeInt[k] + nodeParentInt[k];
        for (uint l = nodes[k].leaf_index; l < nodes[k].leaf_index + nodes[k].leaf_count; ++l)
            nodeFieldIdx[l + 1] = nodeFieldIdx[l] + nf;
    }
    std::vector<leaf_field_t> leafFields(leafFieldIdx[n] + 1);
    std::vector<node_field_t> nodeFields(nodeFieldIdx[n] + 1);
    std::memset(leafFields.data(), 0, sizeof(leaf_field_t) * leafFields.size());
    std::memset(nodeFields.data(), 0, sizeof(node_field_t) * nodeFields.size());

    /* K6 leaf fields (8x8 groups), K7 node fields (local size >= any target leaf_count) */
    launch2(8 * (leafI.size() ? leafI.size() : 1), 8, 8, 8, [&] {
        compute_leaf_interaction_fields((uint)n, leafs.data(), leafFieldIdx.data(), (uint)nn, nodes.data(),
                                        maxLeafCount.data(), (uint)leafI.size(), leafI.data(),
                                        (uint)(leafFields.size() - 1), leafFields.data());
    });
    size_t L = 1;
    for (const interaction_t& it : nodeI) {
        L = std::max<size_t>(L, nodes[it.node_a_index].leaf_count);
        L = std::max<size_t>(L, nodes[it.node_b_index].leaf_count);
    }
    launch1(2 * (nodeI.size() ? nodeI.size() : 1) * L, L, [&] {
        compute_node_interaction_fields((uint)n, nodeFieldIdx.data(), (uint)nn, nodes.data(), nodeParentInt.data(),
                                        (uint)nodeI.size(), nodeI.data(), (uint)(nodeFields.size() - 1),
                                        nodeFields.data());
    });

    /* K8/K9 per-leaf reductions */
    std::vector<force_t> leafForces(n), nodeForces(n);
    {
        size_t local = 64, groups = n / local + (n % local != 0);
        launch1(groups * local, local, [&] {
            convert_leaf_fields_to_forces((uint)n, leafs.data(), leafFieldIdx.data(), leafForces.data(),
                                          (uint)(leafFields.size() - 1), leafFields.data());
        });
        launch1(groups * local, local, [&] {
            convert_node_fields_to_forces((uint)n, leafs.data(), nodeFieldIdx.data(), nodeForces.data(),
                                          (uint)(nodeFields.size() - 1), nodeFields.data());
        });
    }

    /* explicit Euler: src/open_cl_simulation.cpp:600-607 */
    for (int i = 0; i < n; ++i) {
        const float lf[3] = {leafForces[i].force.x, leafForces[i].force.y, leafForces[i].force.z};
        const float nf[3] = {nodeForces[i].force.x, nodeForces[i].force.y, nodeForces[i].force.z};
        for (int d = 0; d < 3; ++d) {
            f_leaf[3 * i + d] = lf[d];
            f_node[3 * i + d] = nf[d];
            float force = lf[d] + nf[d];
            float v = vel3[3 * i + d];
            pos_out[3 * i + d] = pos3[3 * i + d] + v * dt;
            vel_out[3 * i + d] = v + force / mass[i] * dt;
        }
    }

    /* interaction lists mapped back to breadth-first node indices */
    *n_leaf_pairs = (int)leafI.size();
    *n_node_pairs = (int)nodeI.size();
    for (size_t k = 0; k < leafI.size(); ++k) {
        leaf_pairs[2 * k] = T.bfs_of_pre[leafI[k].node_a_index];
        leaf_pairs[2 * k + 1] = T.bfs_of_pre[leafI[k].node_b_index];
    }
    for (size_t k = 0; k < nodeI.size(); ++k) {
        node_pairs[2 * k] = T.bfs_of_pre[nodeI[k].node_a_index];
        node_pairs[2 * k + 1] = T.bfs_of_pre[nodeI[k].node_b_index];
    }
    return 0;
}
