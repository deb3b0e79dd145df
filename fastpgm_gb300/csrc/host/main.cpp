// Command line of the GPU PC-stable engine, option-compatible with the
// reference's `-j 0 -m 0` structure-learning job (src/fastpgm/main.cpp:20-57,
// src/fastpgm/Parameter.cpp:39-83).
//
//   fastpgm -j 0 -m 0 [-t threads] [-g group] [-a alpha] [-f2 train.csv] [-f1 ref.bif] [-ss 0|1]
//           [-e 0|1]   engine: 0 batched device engine (default), 1 plain one-launch-per-test
//
// A relative -f1/-f2 path is taken under the dataset root, like the reference:
// $FASTPGM_DATASET_DIR if set, else ./dataset/ ; a path that exists as given is used as is.
// -j 1 -m 0 (PC-stable + maximum likelihood parameters, -sp 0|1) is provided too.  Other
// jobs of the reference (-j 2..5: inference, ...) are not part of this engine and exit with
// a message.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <sys/stat.h>

#include "fastpgm_gb300_cxx.h"

using std::cout;
using std::endl;
using std::string;

namespace {
struct Parameter {  // defaults of Parameter.cpp:6-37 that the structure-learning job reads
    int job = 0, method = 0, num_threads = 1, verbose = 1, group_size = 1, engine = 0;
    double alpha = 0.05;
    bool save_struct = true, save_param = true;
    string ref_net_file, train_set_file = "alarm/alarm_s5000";
};

void help() {
    cout << "\nUsage: ./fastpgm [command-line options]\n\n"
         << "-h\tPrint this help message\n"
         << "-t\tSpecify number of threads, default 1 (accepted; the GPU engine does not use it)\n"
         << "-j & -m\tSpecify the job & method\n\t-j 0: Structure learning\n\t\t-m 0: PC-Stable\n"
         << "-g\tSpecify group size, default 1 [PC-stable] (accepted; results do not depend on it)\n"
         << "-a\tSpecify significance level alpha, default 0.05 [PC-stable]\n"
         << "-ss\tWhether to output the learned structure, 0 for no, 1 for yes, default 1\n"
         << "-f1\tProvide relative path of reference BN file\n"
         << "-f2\tProvide relative path of training set file, default alarm/alarm_s5000\n"
         << "-e\tEngine: 0 batched device engine (default), 1 plain one-launch-per-test\n";
}

// Parameter.cpp:39-83, including its quirk that "-s?" falls through into "-f?"
void parse(Parameter &p, int argc, char **argv) {
    int i;
    for (i = 1; i < argc && argv[i][0] == '-'; i++) {
        auto need = [&](void) -> const char * {
            if (i + 1 >= argc) {
                printf("\n Missing value for option %s!\n", argv[i]);
                exit(0);
            }
            return argv[++i];
        };
        switch (argv[i][1]) {
            case 'h': help(); exit(0);
            case 'j': p.job = atoi(need()); break;
            case 'm': p.method = atoi(need()); break;
            case 't': p.num_threads = atoi(need()); break;
            case 'q': need(); break;
            case 'g': p.group_size = atoi(need()); break;
            case 'a': p.alpha = std::stod(need()); break;
            case 'c': need(); break;
            case 'e': p.engine = atoi(need()); break;
            case 's':
                switch (argv[i][2]) {
                    case 's': if (atoi(need()) == 0) p.save_struct = false; break;
                    case 'p': if (atoi(need()) == 0) p.save_param = false; break;
                }
                [[fallthrough]];  // as the reference's switch does
            case 'f':
                switch (argv[i][2]) {
                    case '0': need(); break;
                    case '1': p.ref_net_file = need(); break;
                    case '2': p.train_set_file = need(); break;
                    case '3': need(); break;
                    case '4': need(); break;
                }
                break;
            default: printf("\n Unrecognized option %s!\n", argv[i]); exit(0);
        }
    }
    if (p.job < 0 || p.job > 5) {
        cout << "\tError! Please give the right value of -j to specify the job" << endl;
        exit(0);
    }
}

string resolve(const string &f) {
    struct stat sb;
    if (f.empty() || f[0] == '/' || stat(f.c_str(), &sb) == 0) return f;
    const char *root = getenv("FASTPGM_DATASET_DIR");
    string r = root ? string(root) : string("dataset");
    if (!r.empty() && r.back() != '/') r += '/';
    return r + f;
}
}  // namespace

int main(int argc, char **argv) {
    Parameter p;
    parse(p, argc, argv);
    if (p.job != 0 && p.job != 1) {
        cout << "\tError! Only -j 0 (PC-stable structure learning) and -j 1 (PC-stable + maximum likelihood "
                "estimation) are provided by the GPU engine" << endl;
        exit(1);
    }
    if (p.job == 1) {  // main.cpp:66-89
        if (p.method != 0) {
            cout << "\tError! We currently only support -a 0 for PC-Stable structure learning + "
                    "maximum likelihood estimation parameter learning" << endl;
            exit(1);
        }
        cout << "==================================================" << endl
             << "Job: PC-stable + maximum likelihood estimation for learning, #threads = " << p.num_threads << endl
             << "\tgroup size = " << p.group_size << endl
             << "\treference BN: " << p.ref_net_file << endl
             << "\tsample set: " << p.train_set_file << endl
             << "==================================================" << endl;
        const string ref = p.ref_net_file.empty() ? string() : resolve(p.ref_net_file);
        BNL_PCStable(p.verbose, p.num_threads, p.group_size, p.alpha, ref, resolve(p.train_set_file), p.save_struct,
                     p.save_param);
        return 0;
    }
    if (p.method != 0) {
        cout << "\tError! We currently only support -a 0 for PC-Stable structure learning" << endl;
        exit(0);
    }
    cout << "==================================================" << endl
         << "Job: PC-stable for structure learning, #threads = " << p.num_threads << endl
         << "\tgroup size = " << p.group_size << endl
         << "\treference BN: " << p.ref_net_file << endl
         << "\tsample set: " << p.train_set_file << endl
         << "==================================================" << endl;
    const string ref = p.ref_net_file.empty() ? string() : resolve(p.ref_net_file);
    const string train = resolve(p.train_set_file);
    if (p.engine == 0) {
        BNSL_PCStable(p.verbose, p.num_threads, p.group_size, p.alpha, ref, train, p.save_struct);
    } else {
        Dataset d;
        d.LoadCSVTrainingData(train, true, 0);
        Network *net = new Network(true);
        PCStable pc(net, p.alpha);
        pc.engine_mode = FPGM_MODE_PLAIN;
        pc.StructLearnCompData(&d, p.group_size, p.num_threads, false, false, p.save_struct, train + "_struct",
                               p.verbose);
    }
    return 0;
}
