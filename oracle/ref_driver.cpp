// oracle/ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A small driver linked against the reference's OWN PC-stable sources
// (compiled in place from the reference tree by oracle/Makefile; nothing of
// the reference is copied here).  It is the pinned oracle: the shipped golden
// file dataset/alarm/alarm_s5000_struct is reproduced by `pc` mode.
//
//   ref_driver pc <csv> <alpha> <threads> <group_size> <depth> <out_prefix> [verbose]
//       Runs exactly what BNSL_PCStable does (fastpgm_api.cpp:18-44):
//       LoadCSVTrainingData(csv, true, 0); PCStable(new Network(true), alpha, depth);
//       StructLearnCompData(d, gs, T, dag=false, add_root=false, save_struct=true, ...)
//       and writes <out_prefix>_struct (the reference's own writer) and
//       <out_prefix>_sepsets ("a b : z1 z2 ..." per removed pair, key order).
//       Prints one line "ref_pc_seconds <s> num_ci_test <n>".
//
//   ref_driver tests <csv> <alpha> <tests_in> <out>
//       For each input line "x y k z1 .. zk" runs the reference's
//       IndependenceTest::IndependenceResult (IndependenceTest.cpp:35-58) and
//       the reference's Counts2D/Counts3D::FillTable (CellTable.cpp:226-291,
//       430-455), and writes "hash df g2 p indep" where hash is FNV-1a-64 over
//       the reference's int32 joint table n[] in its own cell order, and df/g2
//       follow IndependenceTest.cpp:94-138 on that table.
//
//   ref_driver shd <csv> <alpha> <bif>     (see run_shd)
//   ref_driver bnl <csv> <alpha> <prefix>  (see run_bnl)
//
//   ref_driver mle <csv> <alpha> <edges_in> <out> [param_file]
//       Builds the network's nodes from the dataset as StructureLearning::AssignNodeInformation
//       does (StructureLearning.cpp:11-33), adds the directed edges "parent child" of
//       <edges_in> with Network::AddDirectedEdge, runs the reference's
//       ParameterLearning::LearnParamsKnowStructCompData (ParameterLearning.cpp:10-109) and
//       writes per node "node k v1..vk : p0 p1 ..." (related variables, node first, then
//       its potentials with %.17g), and with param_file the reference's SaveBNParameter file.
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>

#include "fastpgm/Dataset.h"
#include "fastpgm/Network.h"
#include "fastpgm/Timer.h"
#include "fastpgm/structure_learning/PCStable.h"
#include "fastpgm/structure_learning/IndependenceTest.h"
#include "fastpgm/structure_learning/CellTable.h"
#include "fastpgm/parameter_learning/ParameterLearning.h"
#include "fastpgm/CustomNetwork.h"
#include "fastpgm/structure_learning/BNSLComparison.h"

static uint64_t fnv1a_i32(const int *v, long n) {
    uint64_t h = 1469598103934665603ull;
    for (long i = 0; i < n; ++i) {
        uint32_t w = (uint32_t)v[i];
        for (int b = 0; b < 4; ++b) {
            h ^= (w >> (8 * b)) & 0xffu;
            h *= 1099511628211ull;
        }
    }
    return h;
}

static int run_pc(int argc, char **argv) {
    if (argc < 8) { fprintf(stderr, "pc: bad args\n"); return 2; }
    std::string csv = argv[2];
    double alpha = atof(argv[3]);
    int threads = atoi(argv[4]);
    int gs = atoi(argv[5]);
    int depth = atoi(argv[6]);
    std::string prefix = argv[7];
    int verbose = argc > 8 ? atoi(argv[8]) : 0;

    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(csv, true, 0);
    Network *net = new Network(true);
    PCStable *pc = new PCStable(net, alpha, depth);
    double t0 = omp_get_wtime();
    pc->StructLearnCompData(d, gs, threads, false, false, true, prefix + "_struct", verbose);
    double t1 = omp_get_wtime();

    std::ofstream out(prefix + "_sepsets");
    for (const auto &kv : pc->sepset) {
        out << kv.first.first << " " << kv.first.second << " :";
        for (int z : kv.second) out << " " << z;
        out << "\n";
    }
    out.close();
    printf("ref_pc_seconds %.6f num_ci_test %d\n", t1 - t0, pc->num_ci_test);
    return 0;
}

// ref_driver shd <csv> <alpha> <bif>: BNSL_PCStable with a reference network
// (fastpgm_api.cpp:18-44): PC-stable as in `pc` mode (one thread), then
// CustomNetwork::LoadBIFFile and BNSLComparison::GetSHD; prints "SHD = <n>".
static int run_shd(int argc, char **argv) {
    if (argc < 5) { fprintf(stderr, "shd: bad args\n"); return 2; }
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(argv[2], true, 0);
    Network *net = new Network(true);
    PCStable *pc = new PCStable(net, atof(argv[3]), 1000);
    pc->StructLearnCompData(d, 1, 1, false, false, false, "", 0);
    CustomNetwork *r_net = new CustomNetwork();
    r_net->LoadBIFFile(argv[4]);
    BNSLComparison comp(r_net, net);
    printf("SHD = %d\n", comp.GetSHD());
    return 0;
}

// ref_driver bnl <csv> <alpha> <out_prefix>: BNL_PCStable without a reference network
// (fastpgm_api.cpp:46-75): PC-stable (one thread) writing <out_prefix>_struct, then
// ParameterLearning with Laplace alpha 1 on the learned graph writing <out_prefix>_param.
static int run_bnl(int argc, char **argv) {
    if (argc < 5) { fprintf(stderr, "bnl: bad args\n"); return 2; }
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(argv[2], true, 0);
    Network *net = new Network(true);
    PCStable *pc = new PCStable(net, atof(argv[3]), 1000);
    const std::string prefix = argv[4];
    pc->StructLearnCompData(d, 1, 1, false, false, true, prefix + "_struct", 0);
    ParameterLearning *pl = new ParameterLearning(net);
    pl->LearnParamsKnowStructCompData(d, 1, true, prefix + "_param", 0);
    return 0;
}

static int run_mle(int argc, char **argv) {
    if (argc < 6) { fprintf(stderr, "mle: bad args\n"); return 2; }
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(argv[2], true, 0);
    const int alpha = atoi(argv[3]);
    Network *net = new Network(true);
    net->num_nodes = d->num_vars;
    for (int i = 0; i < net->num_nodes; ++i) {  // as StructureLearning::AssignNodeInformation
        DiscreteNode *node = new DiscreteNode(i);
        node->node_name = d->vec_var_names.size() == (size_t)net->num_nodes ? d->vec_var_names[i] : std::to_string(i);
        node->possible_values_ids = d->vars_possible_values_ids[i];
        node->SetDomainSize(d->num_of_possible_values_of_disc_vars[i]);
        net->map_idx_node_ptr[i] = node;
    }
    std::ifstream in(argv[4]);
    int p, c;
    while (in >> p >> c) net->AddDirectedEdge(p, c);
    ParameterLearning *pl = new ParameterLearning(net);
    const bool save = argc > 6;  // optional: the reference's own SaveBNParameter file
    pl->LearnParamsKnowStructCompData(d, alpha, save, save ? argv[6] : "", 0);
    FILE *out = fopen(argv[5], "w");
    if (!out) return 1;
    for (int i = 0; i < net->num_nodes; ++i) {
        const PotentialTableBase &pt = net->pts[i];
        fprintf(out, "%d %d", i, pt.num_variables);
        for (int v : pt.vec_related_variables) fprintf(out, " %d", v);
        fprintf(out, " :");
        for (double x : pt.potentials) fprintf(out, " %.17g", x);
        fprintf(out, "\n");
    }
    fclose(out);
    return 0;
}

static int run_tests(int argc, char **argv) {
    if (argc < 6) { fprintf(stderr, "tests: bad args\n"); return 2; }
    std::string csv = argv[2];
    double alpha = atof(argv[3]);
    Dataset *d = new Dataset();
    d->LoadCSVTrainingData(csv, true, 0);
    std::ifstream in(argv[4]);
    FILE *out = fopen(argv[5], "w");
    Timer timer;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::istringstream ss(line);
        int x, y, k;
        ss >> x >> y >> k;
        std::vector<int> z(k);
        for (int i = 0; i < k; ++i) ss >> z[i];
        int dx = d->num_of_possible_values_of_disc_vars[x];
        int dy = d->num_of_possible_values_of_disc_vars[y];

        uint64_t h;
        int df = 0;
        double g2 = 0.0;
        if (k == 0) {
            Counts2D t(dx, dy, x, y);
            t.FillTable(d, &timer);
            h = fnv1a_i32(t.n, (long)dx * dy);
            int alx = 0, aly = 0;
            for (int i = 0; i < dx; ++i) alx += t.ni[i] > 0;
            for (int j = 0; j < dy; ++j) aly += t.nj[j] > 0;
            alx = alx >= 1 ? alx : 1;
            aly = aly >= 1 ? aly : 1;
            df = (alx - 1) * (aly - 1);
            long total = d->num_instance;
            for (int i = 0; i < dx; ++i) {
                long r = t.ni[i];
                if (r == 0) continue;
                for (int j = 0; j < dy; ++j) {
                    long c = t.nj[j], o = t.n[i * dy + j];
                    if (c == 0 || o == 0) continue;
                    double e = (double)c * (double)r / (double)total;
                    g2 += 2.0 * o * log(o / e);
                }
            }
        } else {
            std::vector<int> dims;
            for (int zi : z) dims.push_back(d->num_of_possible_values_of_disc_vars[zi]);
            Counts3D t(dx, dy, x, y, dims, z);
            t.FillTable(d, &timer);
            h = fnv1a_i32(t.n, (long)t.dimz * dx * dy);
            for (int kk = 0; kk < t.dimz; ++kk) {
                int alx = 0, aly = 0;
                for (int i = 0; i < dx; ++i) alx += t.ni[kk * dx + i] > 0;
                for (int j = 0; j < dy; ++j) aly += t.nj[kk * dy + j] > 0;
                alx = alx >= 1 ? alx : 1;
                aly = aly >= 1 ? aly : 1;
                df += (alx - 1) * (aly - 1);
                long total = t.nk[kk];
                if (total == 0) continue;
                for (int i = 0; i < dx; ++i) {
                    long r = t.ni[kk * dx + i];
                    if (r == 0) continue;
                    for (int j = 0; j < dy; ++j) {
                        long c = t.nj[kk * dy + j], o = t.n[kk * dx * dy + i * dy + j];
                        if (c == 0 || o == 0) continue;
                        double e = (double)c * (double)r / (double)total;
                        g2 += 2.0 * o * log(o / e);
                    }
                }
            }
        }
        IndependenceTest it(d, alpha);
        IndependenceTest::Result r = it.IndependenceResult(x, y, z, "g square", &timer, 1);
        fprintf(out, "%016llx %d %.17g %.17g %d\n", (unsigned long long)h, df, g2, r.p_value,
                r.is_independent ? 1 : 0);
    }
    fclose(out);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_driver pc|tests ...\n"); return 2; }
    std::string mode = argv[1];
    if (mode == "mle") return run_mle(argc, argv);
    if (mode == "shd") return run_shd(argc, argv);
    if (mode == "bnl") return run_bnl(argc, argv);
    if (mode == "pc") return run_pc(argc, argv);
    if (mode == "tests") return run_tests(argc, argv);
    fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
