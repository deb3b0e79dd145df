// C++ drop-in for the reference's PC-stable structure-learning classes and
// the BNSL_PCStable job, driving the GPU engine through the C ABI.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <mutex>
#include <omp.h>
#include <queue>
#include <random>
#include <string_view>

#include "fastpgm_gb300.h"
#include "fastpgm_gb300_cxx.h"
#include "orient.h"
#include "../engine_internal.h"

using std::cout;
using std::endl;
using std::string;
using std::vector;

// ------------------------------------------------------------------ Node / Edge / Network
Node::Node(int index) : Node(index, std::to_string(index)) {}
Node::Node(int index, string name) : node_index(index), node_name(std::move(name)) {}

Edge::Edge(Node *n1, Node *n2, EndPoint e1, EndPoint e2) : node1(n1), node2(n2), end_point1(e1), end_point2(e2) {}

Edge::Edge(Node *n1, Node *n2) {  // Edge.cpp:17-34
    if (n1->GetNodeIndex() < n2->GetNodeIndex()) {
        node1 = n1;
        node2 = n2;
    } else {
        node1 = n2;
        node2 = n1;
    }
    end_point1 = end_point2 = TAIL;
}

Network::Network() : Network(true) {}
Network::Network(bool pure_disc) : pure_discrete(pure_disc) {}
Network::~Network() {
    for (auto &kv : map_idx_node_ptr) delete kv.second;
}

Node *Network::FindNodePtrByIndex(const int &index) const {
    if (index < 0 || index >= num_nodes) {
        fprintf(stderr, "Error in function %s! \nInvalid index [%d]!", __FUNCTION__, index);
        exit(1);
    }
    return map_idx_node_ptr.at(index);
}

std::set<int> Network::GetParentIdxesOfNode(int node_index) { return FindNodePtrByIndex(node_index)->set_parent_indexes; }
std::set<int> Network::GetChildrenIdxesOfNode(int node_index) { return FindNodePtrByIndex(node_index)->set_children_indexes; }

std::vector<int> Network::GetTopoOrd() {  // Network.cpp:371-411 + common.cpp TopoSortOfDAGZeroInDegreeFirst
    if (!topo_ord.empty()) return topo_ord;
    vector<int> indeg(num_nodes, 0);
    for (int v = 0; v < num_nodes; ++v)
        for (int c : FindNodePtrByIndex(v)->set_children_indexes) indeg[c]++;
    std::queue<int> q;
    for (int i = 0; i < num_nodes; ++i)
        if (indeg[i] == 0) q.push(i);
    while (!q.empty()) {
        int u = q.front();
        for (int c : FindNodePtrByIndex(u)->set_children_indexes)
            if (--indeg[c] == 0) q.push(c);
        topo_ord.push_back(u);
        q.pop();
    }
    return topo_ord;
}

void Network::PrintEdges() {
    for (int i = 0; i < num_edges && i < (int)vec_edges.size(); ++i) {
        Edge &e = vec_edges[i];
        cout << i << ": ";
        if (!e.IsDirected())
            cout << e.node1->node_name << " (" << e.node1->GetNodeIndex() << ") -- " << e.node2->node_name << " ("
                 << e.node2->GetNodeIndex() << ")" << endl;
        else if (e.end_point1 == TAIL)
            cout << e.node1->node_name << " (" << e.node1->GetNodeIndex() << ") -> " << e.node2->node_name << " ("
                 << e.node2->GetNodeIndex() << ")" << endl;
        else
            cout << e.node2->node_name << " (" << e.node2->GetNodeIndex() << ") -> " << e.node1->node_name << " ("
                 << e.node1->GetNodeIndex() << ")" << endl;
    }
    cout << "num nodes = " << num_nodes << endl << "num edges = " << num_edges << endl;
}

// ------------------------------------------------------------------ Dataset
namespace {
string trim_right(string s) {  // common.cpp TrimRight
    while (!s.empty() && (unsigned char)s.back() < 33) s.pop_back();
    return s;
}
vector<string> split_commas(const string &s) {  // common.cpp Split
    vector<string> r;
    size_t b = 0, e;
    while ((e = s.find(',', b)) != string::npos) {
        r.push_back(s.substr(b, e - b));
        b = e + 1;
    }
    r.push_back(s.substr(b));
    return r;
}
}  // namespace

namespace {
// Parallel CSV reading with the reference's semantics (Dataset.cpp:389-503): header = names,
// each non-empty line (trailing characters below '!' trimmed) split at commas, and per
// column the state ids in order of first appearance.  Threads parse contiguous row ranges
// with their own per-column value lists (value, first row); the lists are then merged so the
// ids follow the first appearance in the whole file, and each thread's ids are remapped.
// Returns the number of rows, or -1 (and *bad_row = 0-based row) for a row with too few
// fields, or -2 (and *bad_col) for a column with more than 255 states.
int64_t parse_rows_parallel(const string &buf, size_t body, int num_vars, vector<unsigned char> &columns,
                            vector<std::map<string, int>> &ids, int64_t *bad_row, int *bad_col) {
    vector<std::pair<size_t, size_t>> rows;  // [begin, end) of each non-empty trimmed line
    for (size_t b = body; b < buf.size();) {
        size_t e = buf.find('\n', b);
        if (e == string::npos) e = buf.size();
        size_t t = e;
        while (t > b && (unsigned char)buf[t - 1] < 33) --t;
        if (t > b) rows.push_back({b, t});
        b = e + 1;
    }
    const int64_t R = (int64_t)rows.size();
    columns.assign((size_t)num_vars * R, 0);
    const int T = std::max(1, omp_get_max_threads());
    const int64_t chunk = (R + T - 1) / T;
    using Seen = vector<std::pair<std::string_view, int64_t>>;  // value, first row
    vector<vector<Seen>> seen(T, vector<Seen>(num_vars));
    vector<int64_t> short_row(T, -1);
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num();
        const int64_t r0 = std::min(R, t * chunk), r1 = std::min(R, r0 + chunk);
        for (int64_t r = r0; r < r1 && short_row[t] < 0; ++r) {
            size_t b = rows[r].first;
            const size_t e = rows[r].second;
            for (int v = 0; v < num_vars; ++v) {
                if (b > e) { short_row[t] = r; break; }
                size_t c = buf.find(',', b);
                if (c == string::npos || c > e) c = e;
                const std::string_view f(buf.data() + b, c - b);
                Seen &sv = seen[t][v];
                size_t k = 0;
                while (k < sv.size() && sv[k].first != f) ++k;
                if (k == sv.size()) sv.push_back({f, r});
                columns[(size_t)v * R + r] = (unsigned char)std::min<size_t>(k, 255);
                b = c + 1;
            }
        }
    }
    for (int t = 0; t < T; ++t)
        if (short_row[t] >= 0) { *bad_row = short_row[t]; return -1; }
    // ids in order of first appearance in the whole file, and each thread's local -> global
    vector<vector<vector<unsigned char>>> remap(T, vector<vector<unsigned char>>(num_vars));
    ids.assign(num_vars, {});
    for (int v = 0; v < num_vars; ++v) {
        std::map<std::string_view, int64_t> first;
        for (int t = 0; t < T; ++t)
            for (auto &x : seen[t][v]) {
                auto it = first.find(x.first);
                if (it == first.end() || x.second < it->second) first[x.first] = x.second;
            }
        if (first.size() > 255) { *bad_col = v; return -2; }
        vector<std::pair<int64_t, std::string_view>> order;
        for (auto &kv : first) order.push_back({kv.second, kv.first});
        std::sort(order.begin(), order.end());
        std::map<std::string_view, int> gid;
        for (size_t k = 0; k < order.size(); ++k) {
            gid[order[k].second] = (int)k;
            ids[v].emplace(string(order[k].second), (int)k);
        }
        for (int t = 0; t < T; ++t)
            for (auto &x : seen[t][v]) remap[t][v].push_back((unsigned char)gid[x.first]);
    }
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num();
        const int64_t r0 = std::min(R, t * chunk), r1 = std::min(R, r0 + chunk);
        for (int v = 0; v < num_vars; ++v) {
            const vector<unsigned char> &m = remap[t][v];
            unsigned char *col = columns.data() + (size_t)v * R;
            for (int64_t r = r0; r < r1; ++r) col[r] = m[col[r]];
        }
    }
    return R;
}
}  // namespace

void Dataset::LoadCSVTrainingData(string data_file_path, bool str_val, int cls_var_id, std::set<int> cont_vars) {
    if (str_val && cont_vars.empty()) {  // the usual case, read in parallel
        FILE *fp = fopen(data_file_path.c_str(), "rb");
        if (!fp) {
            fprintf(stderr, "Error in function %s!", __FUNCTION__);
            fprintf(stderr, "Unable to open file %s!", data_file_path.c_str());
            exit(1);
        }
        string buf;
        char chunk[1 << 16];
        fseek(fp, 0, SEEK_END);
        const long size = ftell(fp);
        fseek(fp, 0, SEEK_SET);
        if (size > 0) buf.reserve((size_t)size);
        for (size_t got; (got = fread(chunk, 1, sizeof chunk, fp)) > 0;) buf.append(chunk, got);
        fclose(fp);
        class_var_index = cls_var_id;
        size_t e = buf.find('\n');
        if (e == string::npos) e = buf.size();
        vec_var_names = split_commas(trim_right(buf.substr(0, e)));
        num_vars = (int)vec_var_names.size();
        if (std::set<string>(vec_var_names.begin(), vec_var_names.end()).size() != vec_var_names.size()) {
            fprintf(stderr, "Error in function [%s]\nDuplicate variable names in header!", __FUNCTION__);
            exit(1);
        }
        int64_t bad_row = -1;
        int bad_col = -1;
        const int64_t R = parse_rows_parallel(buf, std::min(buf.size(), e + 1), num_vars, columns,
                                              vars_possible_values_ids, &bad_row, &bad_col);
        if (R == -1) {
            fprintf(stderr, "Error in function %s!\nRow %lld has fewer than %d fields.", __FUNCTION__,
                    (long long)bad_row + 2, num_vars);
            exit(1);
        }
        if (R == -2) {
            fprintf(stderr, "Error in function %s!\nVariable %s has more than 255 states; the GPU engine "
                    "stores states as uint8.", __FUNCTION__, vec_var_names[bad_col].c_str());
            exit(1);
        }
        num_instance = (int)R;
        num_of_possible_values_of_disc_vars.resize(num_vars);
        for (int v = 0; v < num_vars; ++v)
            num_of_possible_values_of_disc_vars[v] = (int)vars_possible_values_ids[v].size();
        cout << "Finish loading training data. Number of instances: " << num_instance
             << ". Number of variables: " << num_vars << "." << endl;
        return;
    }
    std::ifstream in(data_file_path);
    if (!in.is_open()) {
        fprintf(stderr, "Error in function %s!", __FUNCTION__);
        fprintf(stderr, "Unable to open file %s!", data_file_path.c_str());
        exit(1);
    }
    if (!cont_vars.empty()) {
        fprintf(stderr, "Error in function %s!\nContinuous variables are not supported by the GPU PC-stable path.",
                __FUNCTION__);
        exit(1);
    }
    class_var_index = cls_var_id;
    string line;
    std::getline(in, line);
    line = trim_right(line);
    vec_var_names = split_commas(line);
    num_vars = (int)vec_var_names.size();
    if (std::set<string>(vec_var_names.begin(), vec_var_names.end()).size() != vec_var_names.size()) {
        fprintf(stderr, "Error in function [%s]\nDuplicate variable names in header!", __FUNCTION__);
        exit(1);
    }
    vars_possible_values_ids.assign(num_vars, {});
    vector<vector<unsigned char>> cols(num_vars);
    while (std::getline(in, line)) {
        line = trim_right(line);
        if (line.empty()) continue;
        vector<string> f = split_commas(line);
        if ((int)f.size() < num_vars) {
            fprintf(stderr, "Error in function %s!\nRow %zu has %zu fields, expected %d.", __FUNCTION__,
                    cols[0].size() + 2, f.size(), num_vars);
            exit(1);
        }
        for (int v = 0; v < num_vars; ++v) {
            int id;
            if (str_val) {  // ids by first appearance (Dataset.cpp:459-467)
                auto &m = vars_possible_values_ids[v];
                auto it = m.find(f[v]);
                if (it == m.end()) {
                    id = (int)m.size();
                    m.emplace(f[v], id);
                } else {
                    id = it->second;
                }
            } else {
                id = std::stoi(f[v]);
                vars_possible_values_ids[v].emplace(f[v], id);
            }
            if (id < 0 || id > 254) {
                fprintf(stderr, "Error in function %s!\nVariable %s has more than 255 states; the GPU engine "
                        "stores states as uint8.", __FUNCTION__, vec_var_names[v].c_str());
                exit(1);
            }
            cols[v].push_back((unsigned char)id);
        }
    }
    num_instance = num_vars ? (int)cols[0].size() : 0;
    num_of_possible_values_of_disc_vars.resize(num_vars);
    columns.resize((size_t)num_vars * num_instance);
    for (int v = 0; v < num_vars; ++v) {
        num_of_possible_values_of_disc_vars[v] = (int)vars_possible_values_ids[v].size();
        std::copy(cols[v].begin(), cols[v].end(), columns.begin() + (size_t)v * num_instance);
    }
    cout << "Finish loading training data. Number of instances: " << num_instance
         << ". Number of variables: " << num_vars << "." << endl;
}

// ------------------------------------------------------------------ StructureLearning
void StructureLearning::AssignNodeInformation(Dataset *dts) {  // StructureLearning.cpp:11-34
    network->num_nodes = dts->num_vars;
    for (int i = 0; i < network->num_nodes; ++i) {
        Node *node = new Node(i);
        if ((int)dts->vec_var_names.size() == network->num_nodes) node->node_name = dts->vec_var_names[i];
        node->possible_values_ids = dts->vars_possible_values_ids[i];
        node->SetDomainSize(dts->num_of_possible_values_of_disc_vars[i]);
        auto it = network->map_idx_node_ptr.find(i);
        if (it != network->map_idx_node_ptr.end()) delete it->second;
        network->map_idx_node_ptr[i] = node;
    }
}

bool StructureLearning::Direct(int a, int c) {  // StructureLearning.cpp:73-84, on the Network records
    Node *pa = network->FindNodePtrByIndex(a), *pc = network->FindNodePtrByIndex(c);
    if (pa->set_children_indexes.count(c) == 0) {
        // refuse an arc that would close a directed cycle
        vector<int> st{c};
        std::set<int> seen{c};
        while (!st.empty()) {
            int u = st.back();
            st.pop_back();
            if (u == a) return false;
            for (int w : network->FindNodePtrByIndex(u)->set_children_indexes)
                if (seen.insert(w).second) st.push_back(w);
        }
        pa->set_children_indexes.insert(c);
        pc->set_parent_indexes.insert(a);
    }
    network->vec_edges.push_back(Edge(pa, pc, TAIL, ARROW));
    Edge und(pa, pc);
    auto it = std::find(network->vec_edges.begin(), network->vec_edges.end(), und);
    if (it != network->vec_edges.end()) network->vec_edges.erase(it);
    return true;
}

vector<int> StructureLearning::FindRootsInDAGForest() {  // StructureLearning.cpp:151-206
    vector<int> roots;
    const int n = network->num_nodes;
    vector<bool> visited(n, false);
    vector<int> indeg(n);
    for (int i = 0; i < n; ++i) indeg[i] = (int)network->GetParentIdxesOfNode(i).size();
    for (;;) {
        int best = -1, root = -1;
        for (int i = 0; i < n; ++i)
            if (indeg[i] == 0 && !visited[i]) {
                int nc = (int)network->GetChildrenIdxesOfNode(i).size();
                if (nc > best) {
                    best = nc;
                    root = i;
                }
            }
        if (best == -1) break;
        visited[root] = true;
        roots.push_back(root);
        std::queue<int> q;
        q.push(root);
        while (!q.empty()) {
            int cur = q.front();
            q.pop();
            for (int c : network->GetChildrenIdxesOfNode(cur))
                if (!visited[c]) { visited[c] = true; q.push(c); }
            for (int p : network->GetParentIdxesOfNode(cur))
                if (!visited[p]) { visited[p] = true; q.push(p); }
        }
    }
    return roots;
}

void StructureLearning::AddRootNode(vector<int> &sub_roots) {  // StructureLearning.cpp:217-236
    Node *root = new Node(network->num_nodes, "ROOT");
    root->possible_values_ids["0"] = 0;
    root->possible_values_ids["1"] = 1;
    root->SetDomainSize(2);
    for (int c : sub_roots) {
        Node *cp = network->FindNodePtrByIndex(c);
        root->set_children_indexes.insert(c);
        cp->set_parent_indexes.insert(root->node_index);
        network->vec_edges.push_back(Edge(root, cp, TAIL, ARROW));
        network->num_edges++;
    }
    network->map_idx_node_ptr[network->num_nodes] = root;
    network->num_nodes++;
}

void StructureLearning::SaveBNStructure(string struct_file) {  // StructureLearning.cpp:238-292
    std::ofstream out(struct_file);
    if (!out.is_open()) {
        fprintf(stderr, "Error in function %s!", __FUNCTION__);
        fprintf(stderr, "Unable to open file %s!", struct_file.c_str());
        exit(1);
    }
    out << "number of nodes = " << network->num_nodes << ", number of edges = " << network->num_edges << "\n";
    if (!network->vec_edges.empty() && network->vec_edges[0].IsDirected()) {
        vector<int> topo = network->GetTopoOrd();
        int k = 0;
        for (int t : topo) {
            Node *tp = network->FindNodePtrByIndex(t);
            for (int c : tp->set_children_indexes)
                out << k++ << ": " << tp->node_name << "/v" << t << " -> " << network->FindNodePtrByIndex(c)->node_name
                    << "/v" << c << "\n";
        }
    } else {
        for (int i = 0; i < network->num_edges && i < (int)network->vec_edges.size(); ++i) {
            Edge &e = network->vec_edges[i];
            Node *a = e.GetNode1(), *b = e.GetNode2();
            out << i << ": ";
            if (!e.IsDirected())
                out << a->node_name << "/v" << a->GetNodeIndex() << " -- " << b->node_name << "/v" << b->GetNodeIndex();
            else if (e.GetEndPoint1() == TAIL)
                out << a->node_name << "/v" << a->GetNodeIndex() << " -> " << b->node_name << "/v" << b->GetNodeIndex();
            else
                out << b->node_name << "/v" << b->GetNodeIndex() << " -> " << a->node_name << "/v" << a->GetNodeIndex();
            out << "\n";
        }
    }
    cout << "Learned structure has been saved in " << struct_file << endl;
}

// ------------------------------------------------------------------ PCStable
namespace {
std::mutex g_engine_mu;
fpgm_engine *g_engines[64] = {nullptr};

int shared_engine(int device, fpgm_engine **out) {
    if (device < 0 || device >= 64) return fpgm::set_error(FPGM_ERR_INVALID, "device %d out of range", device);
    std::lock_guard<std::mutex> lk(g_engine_mu);
    if (!g_engines[device]) {
        int rc = fpgm_engine_create(device, &g_engines[device]);
        if (rc != FPGM_OK) return rc;
    }
    *out = g_engines[device];
    return FPGM_OK;
}

void die_on(int rc) {
    if (rc != FPGM_OK) {
        fprintf(stderr, "Error: %s\n", fpgm_last_error());
        exit(1);
    }
}
}  // namespace

PCStable::PCStable(Network *net, double a, int d) : alpha(a) {  // PCStable.cpp:7-12
    network = net;
    num_ci_test = 0;
    depth = d;
}

PCStable::~PCStable() {  // PCStable.cpp:14-16
    delete network;
    network = nullptr;
}

int PCStable::Run(Dataset *dts, bool dag, bool add_root, bool save_struct, const string &struct_file, int verbose) {
    if (!(alpha >= 0.0 && alpha <= 1.0))
        return fpgm::set_error(FPGM_ERR_INVALID, "Function [IndependenceTest]: Error with incorrect significance level alpha!");
    if (dts->num_vars < 2 || dts->num_instance < 1)
        return fpgm::set_error(FPGM_ERR_INVALID, "PCStable: the dataset needs at least 2 variables and 1 sample");
    const auto t0 = std::chrono::steady_clock::now();
    AssignNodeInformation(dts);
    const int n = network->num_nodes;
    fpgm_engine *eng = nullptr;
    int rc = shared_engine(device, &eng);
    if (rc != FPGM_OK) return rc;
    rc = fpgm_dataset_upload(eng, dts->columns.data(), n, dts->num_instance, 0, nullptr);
    if (rc != FPGM_OK) return rc;
    if (verbose > 0)
        cout << "--------------------------------------------------\n"
             << "Removing edges level by level..." << endl;
    rc = fpgm_pc_skeleton(eng, alpha, depth, engine_mode, &stats);
    if (rc != FPGM_OK) return rc;
    int32_t nn = 0, nr = 0;
    int64_t nv = 0;
    fpgm_pc_result_sizes(eng, &nn, &nr, &nv);
    vector<uint8_t> adj((size_t)n * n);
    vector<int32_t> removed((size_t)nr * 2 + 2), off((size_t)nr + 1), vars((size_t)nv + 1);
    fpgm_pc_result_fetch(eng, adj.data(), removed.data(), off.data(), vars.data());
    int64_t tests = 0;
    for (int l = 0; l < stats.n_levels; ++l) {
        tests += stats.tests[l];
        if (verbose > 0)
            cout << "Level " << l << "... " << endl
                 << "# of CI-tests is " << tests << endl
                 << "# remaining edges = " << stats.edges_after[l] << ", time = " << stats.ms[l] / 1000.0 << endl;
    }
    num_ci_test = (int)tests;
    sepset.clear();
    for (int k = 0; k < nr; ++k)
        sepset[{removed[2 * k], removed[2 * k + 1]}] = std::set<int>(vars.begin() + off[k], vars.begin() + off[k + 1]);
    const auto t1 = std::chrono::steady_clock::now();

    // orientation (PCStable.cpp:240-255)
    if (verbose > 0)
        cout << "--------------------------------------------------\n"
             << "Orienting v-structure and other undirected edges" << endl;
    fpgm::Orienter o(n, adj.data());
    for (int k = 0; k < nr; ++k)
        o.set_sepset(removed[2 * k], removed[2 * k + 1], vars.data() + off[k], off[k + 1] - off[k]);
    o.orient();
    network->vec_edges.clear();
    for (auto &kv : network->map_idx_node_ptr) {
        kv.second->set_parent_indexes.clear();
        kv.second->set_children_indexes.clear();
    }
    for (int v = 0; v < n; ++v)
        for (int c : o.children(v)) {
            network->FindNodePtrByIndex(v)->set_children_indexes.insert(c);
            network->FindNodePtrByIndex(c)->set_parent_indexes.insert(v);
        }
    for (const fpgm::EdgeRec &r : o.edges()) {
        Node *a = network->FindNodePtrByIndex(r.n1), *b = network->FindNodePtrByIndex(r.n2);
        network->vec_edges.push_back(r.directed ? Edge(a, b, TAIL, ARROW) : Edge(a, b));
    }
    network->num_edges = o.num_skeleton_edges();
    if (dag) {  // StructureLearning.cpp:110-144
        std::mt19937 gen(std::random_device{}());
        std::uniform_int_distribution<int> coin(0, 1);
        for (size_t i = 0; i < network->vec_edges.size();) {
            Edge &e = network->vec_edges[i];
            if (e.IsDirected()) break;
            int x = e.node1->GetNodeIndex(), y = e.node2->GetNodeIndex();
            bool ok = coin(gen) == 0 ? (Direct(x, y) || Direct(y, x)) : (Direct(y, x) || Direct(x, y));
            if (!ok) return fpgm::set_error(FPGM_ERR_INVALID, "Error: randomly directing causes loop anyway.");
        }
    }
    const auto t2 = std::chrono::steady_clock::now();
    if (add_root) {
        cout << "--------------------------------------------------\n"
             << "Handling multiple independent sub-graphs...\nFinding roots for sub-graphs and adding the ROOT... "
             << endl;
        vector<int> roots = FindRootsInDAGForest();
        AddRootNode(roots);
        cout << "roots: ";
        for (int r : roots) cout << r << ", ";
        cout << endl;
    }
    if (save_struct) SaveBNStructure(struct_file);
    if (verbose > 0) {
        const double total = std::chrono::duration<double>(t2 - t0).count();
        const double skel = std::chrono::duration<double>(t1 - t0).count();
        cout << "--------------------------------------------------\n"
             << "# of CI-tests = " << num_ci_test << endl
             << "pc-stable step 1: " << skel << " s " << endl
             << " (" << skel / total * 100 << "%)" << endl;
    }
    cout << "pc-stable: " << std::chrono::duration<double>(t2 - t0).count() << " s " << endl;
    return FPGM_OK;
}

void PCStable::StructLearnCompData(Dataset *dts, int group_size, int num_threads, bool dag, bool add_root,
                                   bool save_struct, string struct_file, int verbose) {
    (void)group_size;
    (void)num_threads;
    if (verbose > 0)
        cout << "--------------------------------------------------\n"
             << "Structure learning with PC-Stable..." << endl;
    die_on(Run(dts, dag, add_root, save_struct, struct_file, verbose));
}

// ------------------------------------------------------------------ job API
namespace {
int bnsl_impl(int verbose, int n_threads, int group_size, double alpha, const string &ref_net, const string &train_set,
              bool save_struct, bool learn_params = false, bool save_param = false) {
    Dataset *trainer = new Dataset();
    trainer->LoadCSVTrainingData(train_set, true, 0);
    Network *network = new Network(true);
    PCStable *bnsl = new PCStable(network, alpha);
    (void)group_size;
    (void)n_threads;
    if (verbose > 0)
        cout << "--------------------------------------------------\n"
             << "Structure learning with PC-Stable..." << endl;
    int rc = bnsl->Run(trainer, false, false, save_struct, train_set + "_struct", verbose);
    if (rc == FPGM_OK) {
        if (!ref_net.empty()) {  // fastpgm_api.cpp:32-38: LoadBIFFile + BNSLComparison::GetSHD
            vector<int32_t> edges;
            for (const Edge &e : network->vec_edges) {
                edges.push_back(e.node1->GetNodeIndex());
                edges.push_back(e.node2->GetNodeIndex());
                edges.push_back(e.end_point2 == ARROW ? 1 : 0);
            }
            if (edges.empty()) edges.assign(3, 0);
            int32_t shd = 0;
            rc = fpgm_shd_bif(ref_net.c_str(), network->num_nodes, edges.data(),
                              (int32_t)network->vec_edges.size(), &shd);
            if (rc == FPGM_OK) cout << "SHD = " << shd << endl;
        } else {
            cout << "There is no reference BN (ground-truth) provided, comparison (showing accuracy) is skipped."
                 << endl;
        }
    }
    if (rc == FPGM_OK && learn_params) {  // fastpgm_api.cpp:70-71: MLE on the learned graph, alpha 1
        ParameterLearning bnpl(network);
        bnpl.LearnParamsKnowStructCompData(trainer, 1, save_param, train_set + "_param", verbose);
    }
    delete trainer;
    bnsl->network = nullptr;  // the reference deletes the network itself and never deletes bnsl
    delete network;
    delete bnsl;
    return rc;
}
}  // namespace

void BNL_PCStable(int verbose, int n_threads, int group_size, double alpha, string ref_net, string train_set,
                  bool save_struct, bool save_param) {  // fastpgm_api.cpp:46-75
    die_on(bnsl_impl(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct, true, save_param));
}

extern "C" int fpgm_bnl_pcstable(int32_t verbose, int32_t n_threads, int32_t group_size, double alpha,
                                 const char *ref_net, const char *train_set, int32_t save_struct, int32_t save_param) {
    if (!train_set) return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_bnl_pcstable: NULL train_set");
    return bnsl_impl(verbose, n_threads, group_size, alpha, ref_net ? ref_net : "", train_set, save_struct != 0, true,
                     save_param != 0);
}

void BNSL_PCStable(int verbose, int n_threads, int group_size, double alpha, string ref_net, string train_set,
                   bool save_struct) {
    die_on(bnsl_impl(verbose, n_threads, group_size, alpha, ref_net, train_set, save_struct));
}

extern "C" int fpgm_bnsl_pcstable(int32_t verbose, int32_t n_threads, int32_t group_size, double alpha,
                                  const char *ref_net, const char *train_set, int32_t save_struct) {
    if (!train_set) return fpgm::set_error(FPGM_ERR_INVALID, "fpgm_bnsl_pcstable: train_set is NULL");
    return bnsl_impl(verbose, n_threads, group_size, alpha, ref_net ? ref_net : "", train_set, save_struct != 0);
}

// ------------------------------------------------------------------ ParameterLearning
void PotentialTableBase::GetConfigValueByTableIndex(const int &table_index, int *config_value) const {
    int a = table_index;  // PotentialTableBase.cpp:1179-1187
    for (int i = 0; i < num_variables; ++i) {
        config_value[i] = a / cum_levels[i];
        a %= cum_levels[i];
    }
}

namespace {
string value_name(const Node *node, int id) {  // DiscreteNode::GetValueNameByIndex
    for (const auto &kv : node->possible_values_ids)
        if (kv.second == id) return kv.first;
    return std::to_string(id);
}
}  // namespace

void ParameterLearning::LearnParamsKnowStructCompData(const Dataset *dts, int alpha, bool save_param,
                                                      string param_file, int verbose) {
    if (verbose > 0)
        cout << "--------------------------------------------------" << '\n'
             << "Parameter learning with maximum likelihood estimation... " << endl
             << "Laplace smoothing param alpha = " << alpha << endl;
    const auto t0 = std::chrono::steady_clock::now();
    const int n = dts->num_vars;
    if (network->num_nodes != n) {
        fprintf(stderr, "Error in function %s! The network has %d nodes and the dataset %d variables (a ROOT node is "
                        "not supported here)\n", __FUNCTION__, network->num_nodes, n);
        exit(1);
    }
    vector<int32_t> off(n + 1, 0), par;
    for (int v = 0; v < n; ++v) {
        const Node *node = network->FindNodePtrByIndex(v);
        for (int p : node->set_parent_indexes) par.push_back(p);  // a set: ascending
        off[v + 1] = (int32_t)par.size();
    }
    if (par.empty()) par.push_back(0);
    fpgm_engine *eng = nullptr;
    die_on(shared_engine(device, &eng));
    die_on(fpgm_dataset_upload(eng, dts->columns.data(), n, dts->num_instance, 0, nullptr));
    vector<int64_t> toff(n + 1);
    die_on(fpgm_mle_cpts(eng, off.data(), par.data(), alpha, toff.data(), nullptr));
    vector<double> pot((size_t)toff[n] + 1);
    die_on(fpgm_mle_cpts(eng, off.data(), par.data(), alpha, toff.data(), pot.data()));
    network->pts.assign(n, PotentialTableBase());
    for (int v = 0; v < n; ++v) {  // PotentialTableBase.cpp:102-130 layout
        PotentialTableBase &pt = network->pts[v];
        pt.num_variables = off[v + 1] - off[v] + 1;
        pt.vec_related_variables.push_back(v);
        for (int k = off[v]; k < off[v + 1]; ++k) pt.vec_related_variables.push_back(par[k]);
        for (int u : pt.vec_related_variables) pt.var_dims.push_back(dts->num_of_possible_values_of_disc_vars[u]);
        pt.cum_levels.assign(pt.num_variables, 1);
        for (int i = pt.num_variables - 2; i >= 0; --i) pt.cum_levels[i] = pt.cum_levels[i + 1] * pt.var_dims[i + 1];
        pt.table_size = (int)(toff[v + 1] - toff[v]);
        pt.potentials.assign(pot.begin() + toff[v], pot.begin() + toff[v + 1]);
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    cout << "parameter_learning: " << secs << " s " << endl;
    if (save_param) SaveBNParameter(param_file);
}

void ParameterLearning::SaveBNParameter(string param_file) {  // ParameterLearning.cpp:111-152
    std::ofstream out_file(param_file);
    if (!out_file.is_open()) {
        fprintf(stderr, "Error in function %s!", __FUNCTION__);
        fprintf(stderr, "Unable to open file %s!", param_file.c_str());
        exit(1);
    }
    for (int i = 0; i < network->num_nodes; ++i) {
        const Node *node = network->FindNodePtrByIndex(i);
        const string head = "P (" + node->node_name + "/v" + std::to_string(i) + "=";
        const PotentialTableBase &pt = network->pts[i];
        if (pt.num_variables == 1) {
            for (int j = 0; j < pt.table_size; ++j)
                out_file << head + value_name(node, j) + "/" + std::to_string(j) + ") = " +
                                std::to_string(pt.potentials[j])
                         << endl;
        } else {
            vector<int> config(pt.num_variables);
            for (int j = 0; j < pt.table_size; ++j) {
                pt.GetConfigValueByTableIndex(j, config.data());
                string prob = head + value_name(node, config[0]) + "/" + std::to_string(config[0]) + " | ";
                for (int k = 1; k < pt.num_variables; ++k) {
                    const Node *par = network->FindNodePtrByIndex(pt.vec_related_variables[k]);
                    prob += par->node_name + "/v" + std::to_string(pt.vec_related_variables[k]) + "=" +
                            value_name(par, config[k]) + "/" + std::to_string(config[k]) + ", ";
                }
                prob.pop_back();
                prob.pop_back();
                out_file << prob + ") = " + std::to_string(pt.potentials[j]) << endl;
            }
        }
    }
    cout << "Learned parameters have been saved in " << param_file << endl;
}
