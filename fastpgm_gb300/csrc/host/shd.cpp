// Structural Hamming distance of a learned PC-stable graph against a reference network
// given as a BIF file -- the accuracy report BNSL_PCStable prints when it gets a
// reference network (fastpgm_api.cpp:32-41).
//
//   BIF structure   CustomNetwork::LoadBIFFile (src/fastpgm/CustomNetwork.cpp:52-203):
//                   nodes numbered in declaration order, parents from the
//                   "probability ( child | parents )" headers; the CPT rows are not needed.
//   DAG -> CPDAG    Network::OrderEdge / Network::FindCompelled (src/fastpgm/Network.cpp:547-690),
//                   Chickering's "Find-Compelled" (1995): reversible edges become undirected.
//   distance        BNSLComparison::GetSHD / GetSHDOneEdge
//                   (src/fastpgm/structure_learning/BNSLComparison.cpp:12-73): the reference is
//                   turned into a CPDAG only when the learned graph's first edge is undirected;
//                   each node pair adds 1 when exactly one graph has an edge there, or when
//                   both do and they differ in (first node, second node, arrow at the second).
#include <algorithm>
#include <cstdint>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "fastpgm_gb300.h"
#include "../engine_internal.h"

namespace {

struct BifStructure {
    std::vector<std::string> names;
    std::vector<std::vector<int>> parents;  // in header order
};

std::vector<std::string> tokens(const std::string &line) {
    std::istringstream in(line);
    std::vector<std::string> out;
    std::string t;
    while (in >> t) out.push_back(t);
    return out;
}

std::string trim_comma(std::string s) {
    while (!s.empty() && s.back() == ',') s.pop_back();
    return s;
}

int load_bif_structure(const std::string &path, BifStructure &bif) {
    std::ifstream in(path);
    if (!in.is_open()) return fpgm::set_error(FPGM_ERR_IO, "Unable to open file %s!", path.c_str());
    std::string line;
    std::getline(in, line);  // "network ... {" and "}": skipped like the reference
    std::getline(in, line);
    std::map<std::string, int> index;
    bool in_probabilities = false;
    while (std::getline(in, line)) {
        const std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        if (!in_probabilities && t[0] == "variable" && t.size() > 1) {
            index[t[1]] = (int)bif.names.size();
            bif.names.push_back(t[1]);
            bif.parents.emplace_back();
            continue;
        }
        if (t[0] == "type" && t.size() > 1 && t[1] != "discrete")
            return fpgm::set_error(FPGM_ERR_UNSUPPORTED, "Contain continuous variable in BN!");
        if (t[0] != "probability") continue;
        in_probabilities = true;
        if (t.size() < 4 || t[1] != "(")
            return fpgm::set_error(FPGM_ERR_INVALID, "%s: error in format (%s)", path.c_str(), line.c_str());
        auto child = index.find(t[2]);
        if (child == index.end())
            return fpgm::set_error(FPGM_ERR_INVALID, "%s: unknown variable %s", path.c_str(), t[2].c_str());
        if (t[3] == ")") continue;  // no parents
        for (size_t pos = 4; pos < t.size() && t[pos] != ")"; ++pos) {
            auto p = index.find(trim_comma(t[pos]));
            if (p == index.end())
                return fpgm::set_error(FPGM_ERR_INVALID, "%s: unknown variable %s", path.c_str(), t[pos].c_str());
            bif.parents[child->second].push_back(p->second);
        }
    }
    return FPGM_OK;
}

// One edge record as the reference's Edge keeps it: node1 -> node2 when directed (node1 the
// parent), else node1 < node2 with no arrow.
struct Rec {
    int a, b;
    bool arrow;
};

// Chickering's Order-Edges and Find-Compelled over the DAG's arcs; returns per arc whether
// it is compelled (true) or reversible (false).
std::vector<bool> compelled_arcs(int n, const std::vector<std::pair<int, int>> &arcs) {
    std::vector<std::set<int>> par(n), chi(n);
    for (auto &e : arcs) {
        par[e.second].insert(e.first);
        chi[e.first].insert(e.second);
    }
    // topological order (zero in-degree first, lowest index first)
    std::vector<int> indeg(n), topo, pos(n);
    for (int v = 0; v < n; ++v) indeg[v] = (int)par[v].size();
    std::set<int> ready;
    for (int v = 0; v < n; ++v)
        if (!indeg[v]) ready.insert(v);
    while (!ready.empty()) {
        const int v = *ready.begin();
        ready.erase(ready.begin());
        pos[v] = (int)topo.size();
        topo.push_back(v);
        for (int c : chi[v])
            if (--indeg[c] == 0) ready.insert(c);
    }
    std::map<std::pair<int, int>, int> id;
    for (size_t i = 0; i < arcs.size(); ++i) id[arcs[i]] = (int)i;
    // Order-Edges: y ascending in the topological order, then its parents x descending
    std::vector<int> order;
    for (int y : topo) {
        std::vector<int> xs(par[y].begin(), par[y].end());
        std::sort(xs.begin(), xs.end(), [&](int u, int w) { return pos[u] > pos[w]; });
        for (int x : xs) order.push_back(id[{x, y}]);
    }
    enum { UNKNOWN, COMPELLED, REVERSIBLE };
    std::vector<int> label(arcs.size(), UNKNOWN);
    for (int e : order) {  // the lowest ordered arc still unknown
        if (label[e] != UNKNOWN) continue;
        const int x = arcs[e].first, y = arcs[e].second;
        bool done = false;
        for (int w : par[x]) {
            if (label[id[{w, x}]] != COMPELLED) continue;
            if (!par[y].count(w)) {  // x -> y and every arc into y: compelled
                for (int p : par[y]) label[id[{p, y}]] = COMPELLED;
                done = true;
                break;
            }
            if (label[id[{w, y}]] == UNKNOWN) label[id[{w, y}]] = COMPELLED;
        }
        if (done) continue;
        bool other = false;  // some z -> y with z != x and z not a parent of x
        for (int z : par[y])
            if (z != x && !par[x].count(z)) other = true;
        const int l = other ? COMPELLED : REVERSIBLE;
        label[e] = l;
        for (int p : par[y])
            if (label[id[{p, y}]] == UNKNOWN) label[id[{p, y}]] = l;
    }
    std::vector<bool> out(arcs.size());
    for (size_t i = 0; i < arcs.size(); ++i) out[i] = label[i] == COMPELLED;
    return out;
}

}  // namespace

extern "C" int fpgm_shd_bif(const char *bif_path, int32_t n, const int32_t *edges, int32_t n_edges, int32_t *shd) {
    if (!bif_path || !shd || (n_edges > 0 && !edges) || n < 1 || n_edges < 0)
        return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_shd_bif: bad argument");
    BifStructure bif;
    int rc = load_bif_structure(bif_path, bif);
    if (rc != FPGM_OK) return rc;
    if ((int)bif.names.size() != n)
        return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_shd_bif: the reference network has %d nodes, the learned %d",
                               (int)bif.names.size(), n);
    std::vector<std::pair<int, int>> arcs;
    for (int c = 0; c < n; ++c)
        for (int p : bif.parents[c]) arcs.push_back({p, c});
    std::map<std::pair<int, int>, Rec> truth, learned;  // keyed by (min, max)
    const bool learned_is_dag = n_edges > 0 && edges[2] != 0;  // the reference's IsDAG: first edge
    std::vector<bool> comp(arcs.size(), true);
    if (!learned_is_dag) comp = compelled_arcs(n, arcs);
    for (size_t i = 0; i < arcs.size(); ++i) {
        const int p = arcs[i].first, c = arcs[i].second;
        const auto key = std::make_pair(std::min(p, c), std::max(p, c));
        if (truth.count(key)) continue;  // the first record of a pair, as Network::GetEdge
        truth[key] = comp[i] ? Rec{p, c, true} : Rec{key.first, key.second, false};
    }
    for (int k = 0; k < n_edges; ++k) {
        const int a = edges[3 * k], b = edges[3 * k + 1];
        if (a < 0 || a >= n || b < 0 || b >= n || a == b)
            return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_shd_bif: edge %d (%d, %d) out of range", k, a, b);
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        if (learned.count(key)) continue;
        learned[key] = edges[3 * k + 2] ? Rec{a, b, true} : Rec{key.first, key.second, false};
    }
    int err = 0;
    for (auto &kv : truth) {
        auto it = learned.find(kv.first);
        if (it == learned.end()) { ++err; continue; }
        const Rec &t = kv.second, &l = it->second;
        err += !(t.a == l.a && t.b == l.b && t.arrow == l.arrow);
    }
    for (auto &kv : learned) err += truth.count(kv.first) == 0;
    *shd = err;
    return FPGM_OK;
}
