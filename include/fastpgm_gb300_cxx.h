// fastpgm_gb300_cxx.h -- C++ drop-in for FastPGM's PC-stable structure-learning interface.
//
// The classes keep the reference's names, constructor/method signatures and
// the public state its callers read, so code written against the reference's
// PC-stable path compiles and links against this library instead.  The CI
// testing runs on the GPU engine behind the C ABI in fastpgm_gb300.h.
//
// Reference declarations mirrored (paths inside the FastPGM tree):
//   Node                include/fastpgm/Node.h            (index, name, parent/child index sets)
//   PotentialTableBase  include/fastpgm/PotentialTableBase.h (potentials, variables, radix)
//   ParameterLearning   include/fastpgm/parameter_learning/ParameterLearning.h
//   Edge, EndPoint      include/fastpgm/Edge.h:13-44      (node1/node2, end points, IsDirected)
//   Network             include/fastpgm/Network.h         (num_nodes, num_edges, vec_edges,
//                                                          map_idx_node_ptr, FindNodePtrByIndex,
//                                                          GetParent/ChildrenIdxesOfNode, GetTopoOrd)
//   Dataset             include/fastpgm/Dataset.h:20-76   (num_instance, num_vars, vec_var_names,
//                                                          num_of_possible_values_of_disc_vars,
//                                                          vars_possible_values_ids, LoadCSVTrainingData)
//   StructureLearning   include/fastpgm/structure_learning/StructureLearning.h:13-35
//   PCStable            include/fastpgm/structure_learning/PCStable.h:61-96
//                       (ctor PCStable(Network*, double, int = 1000); StructLearnCompData with the
//                        .cpp parameter order (dag, add_root, save_struct), PCStable.cpp:25-26;
//                        depth, num_ci_test, alpha, sepset)
//   BNSL_PCStable       include/fastpgm/fastpgm_api/fastpgm_api.h:23-25
//
// Differences a caller can observe:
//   * Dataset keeps samples as uint8 (at most 255 states per variable) in
//     `columns`, column-major; the reference's int** dataset_columns is not built.
//   * num_ci_test is the deterministic sequential (group size 1) test count;
//     the reference's counter depends on group size and races under OpenMP.
//   * group_size and num_threads are accepted; neither changes the result.
#ifndef FASTPGM_GB300_CXX_H
#define FASTPGM_GB300_CXX_H

#include <map>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "fastpgm_gb300.h"

enum EndPoint { ARROW, TAIL };

class Node {
public:
    int node_index = 0;
    std::string node_name;
    bool is_discrete = true;
    std::set<int> set_parent_indexes;
    std::set<int> set_children_indexes;
    std::map<std::string, int> possible_values_ids;

    explicit Node(int index);
    Node(int index, std::string name);
    int GetNodeIndex() const { return node_index; }
    void SetDomainSize(int n) { num_potential_vals = n; }
    int GetDomainSize() const { return num_potential_vals; }
    bool HasParents() const { return !set_parent_indexes.empty(); }
    bool IsParentOfThisNode(Node *node_ptr) const { return set_parent_indexes.count(node_ptr->node_index) != 0; }
    bool IsChildOfThisNode(Node *node_ptr) const { return set_children_indexes.count(node_ptr->node_index) != 0; }

private:
    int num_potential_vals = 0;
};

class Edge {
public:
    Node *node1 = nullptr;
    Node *node2 = nullptr;
    EndPoint end_point1 = TAIL;
    EndPoint end_point2 = TAIL;
    bool need_remove = false;

    Edge() {}
    Edge(Node *node1, Node *node2, EndPoint end_point1, EndPoint end_point2);  // directed
    Edge(Node *node1, Node *node2);                                            // undirected, min index first
    bool operator==(const Edge &e) const {
        return node1 == e.node1 && node2 == e.node2 && end_point1 == e.end_point1 && end_point2 == e.end_point2;
    }
    Node *GetNode1() { return node1; }
    Node *GetNode2() { return node2; }
    EndPoint GetEndPoint1() { return end_point1; }
    EndPoint GetEndPoint2() { return end_point2; }
    bool IsDirected() {
        return (end_point1 == ARROW && end_point2 == TAIL) || (end_point1 == TAIL && end_point2 == ARROW);
    }
};

// include/fastpgm/PotentialTableBase.h: the fields parameter learning fills
class PotentialTableBase {
public:
    std::vector<double> potentials;
    std::vector<int> vec_related_variables;  // the node, then its parents ascending
    std::vector<int> var_dims;
    std::vector<int> cum_levels;             // mixed radix, last variable fastest
    int num_variables = 0;
    int table_size = 0;
    void GetConfigValueByTableIndex(const int &table_index, int *config_value) const;
};

class Network {
public:
    std::vector<PotentialTableBase> pts;  // one per node after parameter learning
    std::string network_name;
    int num_nodes = 0;
    int num_edges = 0;
    bool pure_discrete = true;
    std::map<int, Node *> map_idx_node_ptr;
    std::vector<Edge> vec_edges;

    Network();
    explicit Network(bool pure_disc);
    ~Network();
    Node *FindNodePtrByIndex(const int &index) const;
    std::set<int> GetParentIdxesOfNode(int node_index);
    std::set<int> GetChildrenIdxesOfNode(int node_index);
    std::vector<int> GetTopoOrd();
    void PrintEdges();

private:
    std::vector<int> topo_ord;
};

class Dataset {
public:
    int num_instance = 0;
    int num_vars = 0;
    int class_var_index = 0;
    std::vector<std::string> vec_var_names;
    std::vector<int> num_of_possible_values_of_disc_vars;
    std::vector<std::map<std::string, int>> vars_possible_values_ids;
    std::vector<unsigned char> columns;  // [var][sample], column-major uint8 state ids

    // Dataset.cpp:389-503: header = names; ids per column by first appearance.
    // cont_vars (continuous columns) are not supported on this path and must be empty.
    void LoadCSVTrainingData(std::string data_file_path, bool str_val = true, int cls_var_id = 0,
                             std::set<int> cont_vars = std::set<int>());
};

class StructureLearning {
public:
    Network *network = nullptr;

    virtual ~StructureLearning() {}
    // group_size and num_threads are used only for PCStable
    virtual void StructLearnCompData(Dataset *dts, int group_size, int num_threads, bool dag, bool add_root,
                                     bool save_struct, std::string struct_file, int verbose) = 0;
    void AssignNodeInformation(Dataset *dts);
    bool Direct(int a, int c);
    std::vector<int> FindRootsInDAGForest();
    void AddRootNode(std::vector<int> &sub_roots);
    void SaveBNStructure(std::string file);
};

class PCStable : public StructureLearning {
public:
    int depth = 1000;
    int num_ci_test = 0;
    double alpha;
    // separating sets keyed by (min index, max index), as PCStable.h:72
    std::map<std::pair<int, int>, std::set<int>> sepset;

    // engine controls (not in the reference): batched device engine or the
    // plain one-launch-per-test path, and the CUDA device.
    int engine_mode = FPGM_MODE_BATCHED;
    int device = 0;
    fpgm_pc_stats stats{};

    PCStable(Network *net, double a, int d = 1000);
    ~PCStable();

    // Parameter order of the reference's definition (PCStable.cpp:25-26).
    virtual void StructLearnCompData(Dataset *dts, int group_size, int num_threads, bool dag, bool add_root,
                                     bool save_struct, std::string struct_file, int verbose);
    // Same work, returning an FPGM status instead of exiting on failure.
    int Run(Dataset *dts, bool dag, bool add_root, bool save_struct, const std::string &struct_file, int verbose);
};

// parameter_learning/ParameterLearning.h:14-23: maximum-likelihood tables with Laplace
// smoothing for the network's known DAG (the parents in Node::set_parent_indexes), counted on
// the GPU (fpgm_mle_cpts).  A virtual ROOT node (add_root) is not supported here.
class ParameterLearning {
public:
    Network *network;
    int device = 0;  // CUDA device (not in the reference)

    explicit ParameterLearning(Network *net) : network(net) {}
    void LearnParamsKnowStructCompData(const Dataset *dts, int alpha, bool save_param, std::string param_file,
                                       int verbose);
    void SaveBNParameter(std::string param_file);
};

// fastpgm_api.cpp:46-75: PC-stable, the SHD report, then maximum-likelihood parameters
// (Laplace alpha 1) for the learned graph, written to train_set + "_param" when save_param.
void BNL_PCStable(int verbose, int n_threads, int group_size, double alpha, std::string ref_net,
                  std::string train_set, bool save_struct, bool save_param);

// fastpgm_api.cpp:18-44
void BNSL_PCStable(int verbose, int n_threads, int group_size, double alpha, std::string ref_net,
                   std::string train_set, bool save_struct);

#endif
