// CPDAG orientation of a PC-stable skeleton, reproducing the reference's
// order-dependent result exactly.
//
// The reference (structure_learning/PCStable.cpp:639-847) orients with a
// vector of edge records whose order is part of the result: directed edges
// are appended at the end, deleted records are erased in place, and the
// Meek-rule pass walks the vector by position and stops at the first record
// that is not undirected.  Parent/child relations are kept apart from the
// records (Network.cpp:169-268, :327-347) and a new arc is refused when the
// relation graph would contain a cycle (ContainCircle, Network.cpp:515-545).
// This class keeps the same two structures -- an edge-record vector with the
// same erase/append semantics and a relation graph -- but answers adjacency
// from an n x n byte matrix and cycle queries with one DFS from the child
// (the relation graph is acyclic before every insertion), so orientation is
// O(E * (n + E)) instead of the reference's O(n^2) per inserted arc.
#pragma once
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace fpgm {

struct EdgeRec {
    int n1, n2;     // directed: n1 -> n2 (tail, arrow); undirected: n1 < n2
    bool directed;
};

class Orienter {
public:
    // skel: n x n skeleton adjacency (symmetric); sepsets keyed by a*n+b (a<b).
    Orienter(int n, const uint8_t *skel);
    void set_sepset(int a, int b, const int32_t *vars, int len);
    // Runs OrientVStructure then OrientImplied (PCStable.cpp:240-250).
    void orient();
    const std::vector<EdgeRec> &edges() const { return vec_edges_; }
    int num_skeleton_edges() const { return num_edges_; }
    bool is_parent(int p, int c) const { return rel_[(size_t)p * n_ + c] != 0; }
    std::vector<int> parents(int v) const;
    std::vector<int> children(int v) const;
    // Kahn order over the relation graph, zero in-degree first, children scanned by index
    // (common.cpp TopoSortOfDAGZeroInDegreeFirst).
    std::vector<int> topo_order() const;
    // Network-style edge operations with the reference's semantics.
    bool add_directed(int p, int c);
    bool delete_directed(int p, int c);
    void add_undirected(int a, int b);
    bool delete_undirected(int a, int b);
    bool direct(int a, int c);
    bool is_undirected(int u, int v) const {
        return skel_[(size_t)u * n_ + v] && !rel_[(size_t)u * n_ + v] && !rel_[(size_t)v * n_ + u];
    }

private:
    void orient_vstructures();
    void orient_implied();
    bool rule1(int b, int c);
    bool rule2(int a, int c);
    bool rule3(int d, int a);
    std::vector<int> common_adjacents(int x, int y) const;
    bool reaches(int from, int to) const;

    int n_;
    int num_edges_ = 0;
    std::vector<uint8_t> skel_;
    std::vector<std::vector<int>> adj_;       // sorted skeleton neighbours
    std::vector<uint8_t> rel_;                // rel_[p*n+c] = 1 if p is a parent of c
    std::vector<std::vector<int>> kids_;      // children lists (unordered) for DFS
    std::vector<EdgeRec> vec_edges_;
    std::unordered_map<int64_t, std::vector<int>> sep_;
    mutable std::vector<int> stack_;
    mutable std::vector<uint32_t> seen_;
    mutable uint32_t stamp_ = 0;
};

// Writes the reference's _struct text (StructureLearning.cpp:238-292).
// num_edges: the skeleton edge count the reference prints and iterates.
bool write_struct(const std::string &path, int n, const std::vector<std::string> &names,
                  const std::vector<EdgeRec> &edges, int num_edges, const Orienter *rel);

}  // namespace fpgm
