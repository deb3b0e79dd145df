// CPDAG orientation with the reference's edge-record semantics (see orient.h).
#include "orient.h"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <queue>

#include "fastpgm_gb300.h"
#include "../engine_internal.h"

namespace fpgm {

Orienter::Orienter(int n, const uint8_t *skel)
    : n_(n), skel_(skel, skel + (size_t)n * n), adj_(n), rel_((size_t)n * n, 0), kids_(n), seen_(n, 0) {
    // skeleton edges in complete-graph order: what is left of vec_edges after
    // the removal passes (PCStable.cpp:179-195, :369-386)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (skel_[(size_t)i * n + j]) {
                adj_[i].push_back(j);
                if (j > i) vec_edges_.push_back({i, j, false});
            }
    num_edges_ = (int)vec_edges_.size();
}

void Orienter::set_sepset(int a, int b, const int32_t *vars, int len) {
    if (a > b) std::swap(a, b);
    std::vector<int> v(vars, vars + len);
    std::sort(v.begin(), v.end());
    sep_[(int64_t)a * n_ + b] = std::move(v);
}

std::vector<int> Orienter::parents(int v) const {
    std::vector<int> p;
    for (int u = 0; u < n_; ++u)
        if (rel_[(size_t)u * n_ + v]) p.push_back(u);
    return p;
}

std::vector<int> Orienter::children(int v) const {
    std::vector<int> c;
    for (int u = 0; u < n_; ++u)
        if (rel_[(size_t)v * n_ + u]) c.push_back(u);
    return c;
}

bool Orienter::reaches(int from, int to) const {
    if (from == to) return true;
    if (++stamp_ == 0) {
        std::fill(seen_.begin(), seen_.end(), 0);
        stamp_ = 1;
    }
    stack_.clear();
    stack_.push_back(from);
    seen_[from] = stamp_;
    while (!stack_.empty()) {
        int u = stack_.back();
        stack_.pop_back();
        for (int w : kids_[u]) {
            if (w == to) return true;
            if (seen_[w] != stamp_) {
                seen_[w] = stamp_;
                stack_.push_back(w);
            }
        }
    }
    return false;
}

// Network::AddDirectedEdge (Network.cpp:169-191): set the relation, refuse it
// if the relation graph now has a cycle, else append a (tail, arrow) record.
bool Orienter::add_directed(int p, int c) {
    const size_t k = (size_t)p * n_ + c;
    if (!rel_[k]) {
        // the relation graph is acyclic before every insertion, so the new arc
        // closes a cycle iff c already reaches p
        if (reaches(c, p)) return false;
        rel_[k] = 1;
        kids_[p].push_back(c);
    }
    vec_edges_.push_back({p, c, true});
    return true;
}

// Network::DeleteDirectedEdge (Network.cpp:193-213)
bool Orienter::delete_directed(int p, int c) {
    for (size_t i = 0; i < vec_edges_.size(); ++i) {
        const EdgeRec &r = vec_edges_[i];
        if (r.directed && r.n1 == p && r.n2 == c) {
            if (rel_[(size_t)p * n_ + c]) {
                rel_[(size_t)p * n_ + c] = 0;
                auto &kv = kids_[p];
                kv.erase(std::find(kv.begin(), kv.end(), c));
            }
            vec_edges_.erase(vec_edges_.begin() + (long)i);
            return true;
        }
    }
    return false;
}

// Network::AddUndirectedEdge (Network.cpp:219-240): append, min index first (Edge.cpp:17-34)
void Orienter::add_undirected(int a, int b) {
    if (a > b) std::swap(a, b);
    vec_edges_.push_back({a, b, false});
}

// Network::DeleteUndirectedEdge (Network.cpp:242-268)
bool Orienter::delete_undirected(int a, int b) {
    if (a > b) std::swap(a, b);
    for (size_t i = 0; i < vec_edges_.size(); ++i) {
        const EdgeRec &r = vec_edges_[i];
        if (!r.directed && r.n1 == a && r.n2 == b) {
            vec_edges_.erase(vec_edges_.begin() + (long)i);
            return true;
        }
    }
    return false;
}

// StructureLearning::Direct (StructureLearning.cpp:73-84)
bool Orienter::direct(int a, int c) {
    bool added = add_directed(a, c);
    if (added) delete_undirected(a, c);
    return added;
}

std::vector<int> Orienter::common_adjacents(int x, int y) const {
    std::vector<int> r;
    std::set_intersection(adj_[x].begin(), adj_[x].end(), adj_[y].begin(), adj_[y].end(), std::back_inserter(r));
    return r;
}

// PCStable::OrientVStructure (PCStable.cpp:639-724)
void Orienter::orient_vstructures() {
    static const std::vector<int> kEmpty;
    for (int b = 0; b < n_; ++b) {
        const std::vector<int> &nb = adj_[b];
        if (nb.size() < 2) continue;
        for (size_t ia = 0; ia + 1 < nb.size(); ++ia)
            for (size_t ic = ia + 1; ic < nb.size(); ++ic) {
                const int a = nb[ia], c = nb[ic];
                if (skel_[(size_t)a * n_ + c]) continue;
                auto it = sep_.find((int64_t)a * n_ + c);
                const std::vector<int> &s = it == sep_.end() ? kEmpty : it->second;
                if (std::binary_search(s.begin(), s.end(), b)) continue;
                bool dd1 = delete_directed(b, a), du1 = false;
                if (!dd1) du1 = delete_undirected(a, b);
                const bool to1 = dd1 || du1;
                bool dd2 = delete_directed(b, c), du2 = false;
                if (!dd2) du2 = delete_undirected(c, b);
                const bool to2 = dd2 || du2;
                bool added1 = false, added2 = false;
                if (to1) added1 = add_directed(a, b);
                if (to2) added2 = add_directed(c, b);
                if ((to1 && !added1) || (to2 && !added2)) {
                    if (to1) {
                        if (dd1) add_directed(b, a); else add_undirected(a, b);
                    }
                    if (to2) {
                        if (dd2) add_directed(b, c); else add_undirected(c, b);
                    }
                }
            }
    }
}

// Rule 1 (PCStable.cpp:777-785): a -> b, b -- c, a not adjacent to c  =>  b -> c
bool Orienter::rule1(int b, int c) {
    for (int a : parents(b)) {
        if (skel_[(size_t)c * n_ + a]) continue;
        if (direct(b, c)) return true;
    }
    return false;
}

// Rule 2 (PCStable.cpp:790-803): a -> b -> c, a -- c  =>  a -> c
bool Orienter::rule2(int a, int c) {
    for (int b : common_adjacents(a, c))
        if (rel_[(size_t)a * n_ + b] && rel_[(size_t)b * n_ + c])
            if (direct(a, c)) return true;
    return false;
}

// Rule 3 (PCStable.cpp:808-847): d--a, d--b, d--c, b->a, c->a, b and c not adjacent  =>  d -> a
bool Orienter::rule3(int d, int a) {
    std::vector<int> com = common_adjacents(a, d);
    if (com.size() < 2) return false;
    for (size_t i = 0; i < com.size(); ++i)
        for (size_t j = i + 1; j < com.size(); ++j) {
            const int b = com[i], c = com[j];
            if (skel_[(size_t)b * n_ + c]) continue;
            if (is_undirected(d, b) && is_undirected(d, c) && rel_[(size_t)b * n_ + a] && rel_[(size_t)c * n_ + a])
                if (direct(d, a)) return true;
        }
    return false;
}

// PCStable::OrientImplied (PCStable.cpp:734-772): walk records by position,
// stay on the position after a rule fires, stop at the first non-undirected pair.
void Orienter::orient_implied() {
    bool oriented = true;
    while (oriented) {
        oriented = false;
        size_t i = 0;
        while (i < vec_edges_.size()) {
            const int x = vec_edges_[i].n1, y = vec_edges_[i].n2;
            if (!is_undirected(x, y)) break;
            if (rule1(x, y) || rule1(y, x) || rule2(x, y) || rule2(y, x) || rule3(x, y) || rule3(y, x))
                oriented = true;
            else
                ++i;
        }
    }
}

void Orienter::orient() {
    orient_vstructures();
    orient_implied();
}

std::vector<int> Orienter::topo_order() const {
    std::vector<int> indeg(n_, 0), out;
    for (int p = 0; p < n_; ++p)
        for (int c = 0; c < n_; ++c) indeg[c] += rel_[(size_t)p * n_ + c];
    std::queue<int> q;
    for (int i = 0; i < n_; ++i)
        if (indeg[i] == 0) q.push(i);
    while (!q.empty()) {
        int u = q.front();
        for (int j = 0; j < n_; ++j)
            if (rel_[(size_t)u * n_ + j] && --indeg[j] == 0) q.push(j);
        out.push_back(u);
        q.pop();
    }
    return out;
}

bool write_struct(const std::string &path, int n, const std::vector<std::string> &names,
                  const std::vector<EdgeRec> &edges, int num_edges, const Orienter *rel) {
    std::ofstream f(path);
    if (!f.is_open()) return false;
    auto name = [&](int v) { return (int)names.size() == n ? names[v] : std::to_string(v); };
    f << "number of nodes = " << n << ", number of edges = " << num_edges << "\n";
    if (!edges.empty() && edges[0].directed) {
        // DAG branch: nodes in topological order, children ascending
        std::vector<int> topo;
        std::vector<std::vector<int>> kids(n);
        if (rel) {
            topo = rel->topo_order();
            for (int v = 0; v < n; ++v) kids[v] = rel->children(v);
        }
        int k = 0;
        for (int t : topo)
            for (int c : kids[t])
                f << k++ << ": " << name(t) << "/v" << t << " -> " << name(c) << "/v" << c << "\n";
    } else {
        for (int i = 0; i < num_edges && i < (int)edges.size(); ++i) {
            const EdgeRec &r = edges[i];
            f << i << ": " << name(r.n1) << "/v" << r.n1 << (r.directed ? " -> " : " -- ") << name(r.n2) << "/v"
              << r.n2 << "\n";
        }
    }
    f.close();
    return !f.fail();
}

}  // namespace fpgm

// ---------------------------------------------------------------- C ABI
extern "C" int fpgm_orient_cpdag(int32_t n, const uint8_t *adj, int32_t n_removed, const int32_t *removed,
                                 const int32_t *sep_offsets, const int32_t *sep_vars, int32_t *out_edges,
                                 int32_t *out_n_edges) {
    if (n < 1 || !adj || !out_edges || !out_n_edges || (n_removed > 0 && (!removed || !sep_offsets)))
        return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_orient_cpdag: bad arguments");
    fpgm::Orienter o(n, adj);
    for (int k = 0; k < n_removed; ++k)
        o.set_sepset(removed[2 * k], removed[2 * k + 1], sep_vars + sep_offsets[k], sep_offsets[k + 1] - sep_offsets[k]);
    o.orient();
    const auto &E = o.edges();
    for (size_t i = 0; i < E.size(); ++i) {
        out_edges[3 * i] = E[i].n1;
        out_edges[3 * i + 1] = E[i].n2;
        out_edges[3 * i + 2] = E[i].directed ? 1 : 0;
    }
    *out_n_edges = (int32_t)E.size();
    return FPGM_OK;
}

extern "C" int fpgm_write_struct(const char *path, int32_t n, const char *const *names, const int32_t *edges,
                                 int32_t n_edges, int32_t num_edges_header) {
    if (!path || n < 1 || (n_edges > 0 && !edges)) return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_write_struct: bad arguments");
    std::vector<std::string> nm;
    if (names)
        for (int i = 0; i < n; ++i) nm.push_back(names[i]);
    std::vector<fpgm::EdgeRec> E((size_t)n_edges);
    // relation graph for the DAG branch: the directed records
    std::vector<uint8_t> none((size_t)n * n, 0);
    fpgm::Orienter rel(n, none.data());
    for (int i = 0; i < n_edges; ++i) {
        E[i] = {edges[3 * i], edges[3 * i + 1], edges[3 * i + 2] != 0};
        if (E[i].directed && !rel.is_parent(E[i].n1, E[i].n2)) rel.add_directed(E[i].n1, E[i].n2);
    }
    if (!fpgm::write_struct(path, n, nm, E, num_edges_header, &rel))
        return fpgm::set_error(FPGM_ERR_IO, "Unable to open file %s!", path);
    return FPGM_OK;
}
