/*
 * fastpgm_gb300.h -- C ABI of the GB300 PC-stable CI-testing engine.
 *
 * Plain pointers and sizes only; every entry point returns an int status
 * (FPGM_OK or a negative FPGM_ERR_*), and fpgm_last_error() gives the
 * calling thread's last message.  The library never exits the process; the
 * C++ drop-in layer (fastpgm_gb300/csrc/host) maps a failure to the
 * reference's "message + exit(1)" behaviour.
 *
 * Reference interfaces each group replaces (paths inside the FastPGM tree):
 *   fpgm_dataset_upload   Dataset::LoadCSVTrainingData id assignment and
 *                         RowMajor2ColumnMajor (src/fastpgm/Dataset.cpp:389-503,
 *                         :459-467, :846-857): column-major data + observed
 *                         cardinalities (include/fastpgm/Dataset.h:29-32)
 *   fpgm_ci_test(_batch)  IndependenceTest::IndependenceResult with the
 *                         "g square" metric (structure_learning/IndependenceTest.cpp:35-58,
 *                         :65-155, :295-364) over Counts2D/Counts3D tables
 *                         (structure_learning/CellTable.cpp:23-72, :226-291, :430-455)
 *   fpgm_pc_skeleton      PCStable::StructLearnByPCStable levels 0..depth-1
 *                         (structure_learning/PCStable.cpp:84-231) with
 *                         SearchAtDepth/CheckEdge/Testing/FreeDegree
 *                         (:265-388, :399-494, :526-614, :620-626)
 *   fpgm_pc_result_*      PCStable::sepset and the skeleton adjacency the
 *                         reference keeps in `adjacencies` (PCStable.h:72, PCStable.cpp:118-127)
 *   fpgm_orient_cpdag     PCStable::OrientVStructure / OrientImplied / Rule1-3
 *                         (PCStable.cpp:639-847) with Network edge bookkeeping
 *                         (src/fastpgm/Network.cpp:169-268, :515-545)
 *   fpgm_bnsl_pcstable    BNSL_PCStable (src/fastpgm/fastpgm_api/fastpgm_api.cpp:18-44,
 *                         include/fastpgm/fastpgm_api/fastpgm_api.h:23-25)
 *   fpgm_generate_network SampleSetGenerator forward sampling
 *                         (src/fastpgm/SampleSetGenerator.cpp), made seedable
 */
#ifndef FASTPGM_GB300_H
#define FASTPGM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FPGM_OK = 0,
    FPGM_ERR_INVALID = -1,      /* bad argument (the reference prints and exits) */
    FPGM_ERR_OOM = -2,          /* device or host allocation failed */
    FPGM_ERR_CUDA = -3,         /* CUDA runtime error */
    FPGM_ERR_TIMEOUT = -4,      /* a bounded device wait gave up */
    FPGM_ERR_IO = -5,           /* file could not be opened / written */
    FPGM_ERR_UNSUPPORTED = -6,  /* input outside the engine's limits (message says which) */
    FPGM_ERR_STATE = -7         /* call out of order (e.g. no dataset uploaded) */
};

enum { FPGM_MODE_BATCHED = 0, FPGM_MODE_PLAIN = 1 };

/* Largest conditioning-set size the engine accepts. */
#define FPGM_MAX_COND 30

typedef struct fpgm_engine fpgm_engine;

typedef struct {
    uint64_t table_hash;   /* FNV-1a-64 of the int32 joint table n[z][x][y] in reference cell order
                              (0 if not asked, and 0 for tests counted by observed strata) */
    uint64_t cell_hash;    /* order-free fingerprint: sum over nonzero cells of a 64-bit mix of
                              (cell index in reference order, count) (0 if not asked) */
    int64_t cells;         /* dz * dx * dy (observed strata * dx * dy on the compact path) */
    int32_t df;            /* adjusted degrees of freedom (IndependenceTest.cpp:96-111) */
    int32_t independent;   /* df == 0 or p > alpha */
    double g2;             /* G^2 the decision used: FP64 when rechecked, else the FP32 compensated sum */
    double p_value;        /* 1 - P(df/2, G^2/2) */
    int32_t rechecked;     /* 1 when G^2 was computed with FP64 terms (recheck band or compact path) */
    int32_t path;          /* 0 warp tier, 1 CTA tier or plain kernel, 2 compact strata,
                              3 partitioned strata, 4 partitioned strata scored by several CTAs */
} fpgm_ci_result;

typedef struct {
    int32_t n_levels;
    int64_t tests[64];           /* tests per level, the reference's sequential group-size-1 count */
    int64_t tests_executed[64];  /* tests actually run (batched mode includes speculative ones) */
    int32_t edges_after[64];     /* skeleton edges left after the level */
    int32_t waves[64];           /* batched waves in the level */
    double ms[64];               /* wall time of the level, host clock around device work */
    int64_t rechecks;            /* tests that entered the FP64 band */
    int64_t near_ties;           /* FP64 |p - alpha| < 1e-12 (decision could differ from any other FP64 order) */
    int64_t large_tests;         /* tests counted in global memory */
    double max_abs_dp;           /* max |p32 - p64| over rechecked tests */
    double count_ms;             /* device time of the shared-memory counting+scoring kernel (CUDA events) */
    double count_bytes;          /* algorithmic bytes its tests read: sum (2+d) * n_samples */
    double large_ms;             /* device time of the global-memory (large table) kernel */
    int64_t count_launches;      /* launches of the counting+scoring kernels */
    int64_t kernel_launches;     /* launches of this library's own kernels (library scans excluded) */
    double span_ms;              /* CUDA-event span of the whole call on the engine's stream */
    double total_ms;             /* host wall time of the whole skeleton call */
    double large_bytes;          /* algorithmic bytes of the global-memory kernel's tests */
    double gram_ms;              /* device time of level 0 on the tensor cores (one-hot build, Gram GEMM,
                                    pair scoring; 0 when level 0 ran on the counting kernels) */
    double gram_flops;           /* tensor-core flops of that Gram GEMM */
    int64_t gram_tests;          /* level-0 tests decided from the Gram matrix */
    int32_t tune_buckets;        /* online autotuner: (samples, |Z|, cells/samples) buckets timed both ways */
    int32_t tune_partition;      /* ... of which the partition kernel is the faster tier-2 method */
    int64_t tune_timed;          /* tier-2 tests timed by the autotuner since the engine was created */
    double graph_ms;             /* host time capturing and instantiating the levels' CUDA graphs */
} fpgm_pc_stats;

typedef struct {
    int32_t n_nodes;
    int32_t n_edges;         /* exact edge count; <= 0 means round(avg_indegree * n_nodes) */
    double avg_indegree;
    int32_t max_indegree;
    int32_t card_min, card_max;   /* uniform cardinality range */
    double tail_frac;             /* with this probability draw from [tail_min, tail_max] instead */
    int32_t tail_min, tail_max;
    double dirichlet_alpha;       /* CPT rows ~ Dirichlet(alpha) */
    int64_t n_samples;
    uint64_t seed;
} fpgm_gen_spec;

/* ---- errors ---- */
const char *fpgm_last_error(void);

/* ---- engine lifetime ---- */
int fpgm_engine_create(int32_t device, fpgm_engine **out);
int fpgm_engine_destroy(fpgm_engine *eng);

/* ---- data ----
 * columns: n_vars x n_samples uint8, column-major (column v at columns + v*n_samples).
 * relabel != 0: ids become first-appearance order per column and cardinality
 * the number of distinct observed values (Dataset.cpp:459-467, :486-488).
 * relabel == 0: values are used as given; out_card (if given) then receives max+1.
 * out_card may be NULL. */
int fpgm_dataset_upload(fpgm_engine *eng, const uint8_t *columns, int32_t n_vars, int64_t n_samples,
                        int32_t relabel, uint8_t *out_card);
/* Several independent datasets in one engine (no counterpart in the reference, which
 * learns one dataset per call): dataset j has job_vars[j] variables of job_samples[j]
 * samples, column-major at job_columns[j].  The engine numbers the variables in dataset
 * order (dataset 0's first, then dataset 1's, ...); fpgm_pc_skeleton then learns every
 * dataset's skeleton at once -- the complete graph within each dataset, never across --
 * with every level's tests of all datasets in the same waves, and its results use that
 * numbering.  CI tests must keep to one dataset.  out_card receives all variables'
 * cardinalities.  At most 65,535 variables in all (16,384 for the batched skeleton). */
int fpgm_dataset_upload_jobs(fpgm_engine *eng, int32_t n_jobs, const int32_t *job_vars, const int64_t *job_samples,
                             const uint8_t *const *job_columns, int32_t relabel, uint8_t *out_card);
/* ---- accuracy against a reference network ----
 * Structural Hamming distance of a learned graph -- edges as fpgm_orient_cpdag returns them,
 * (a, b, directed) in the reference's record order -- against the network of a BIF file, as
 * BNSL_PCStable reports it (fastpgm_api.cpp:32-41: CustomNetwork::LoadBIFFile,
 * BNSLComparison::GetSHD, structure_learning/BNSLComparison.cpp:12-73): when the learned
 * graph's first edge is undirected, the reference DAG is first turned into its CPDAG
 * (Network::OrderEdge/FindCompelled, Network.cpp:547-690). */
int fpgm_shd_bif(const char *bif_path, int32_t n_nodes, const int32_t *edges, int32_t n_edges, int32_t *shd);

/* ---- parameter learning for a known DAG ----
 * Maximum-likelihood tables with Laplace smoothing alpha over the uploaded data, as
 * ParameterLearning::LearnParamsKnowStructCompData (src/fastpgm/parameter_learning/
 * ParameterLearning.cpp:10-109, job -j 1 of the reference's command line): node v's table is
 * over (v, its parents ascending), v's state slowest, parent configurations in mixed radix with
 * the last parent fastest (PotentialTableBase.cpp:102-130), and
 *   potentials[table_off[v] + j] = (N[j] + alpha) / (N(parents of j) + alpha * card[v]).
 * parent_off[n_vars+1] / parents: each node's parents, ascending, no repeats, from its own
 * dataset.  table_off[n_vars+1] is always filled; potentials (table_off[n_vars] doubles) only
 * when not NULL, so a first call with NULL sizes the buffer.  Tables beyond 2^30 entries:
 * FPGM_ERR_UNSUPPORTED. */
int fpgm_mle_cpts(fpgm_engine *eng, const int32_t *parent_off, const int32_t *parents, int32_t alpha,
                  int64_t *table_off, double *potentials);

/* Copies the (relabelled) device columns back, n_vars*n_samples bytes (one dataset only). */
int fpgm_dataset_download(fpgm_engine *eng, uint8_t *columns);

/* ---- single / batched CI tests (G^2) ----
 * fpgm_ci_test: one test, one kernel launch ("plain" path; a joint table beyond the
 * shared-memory tiers runs the three tier-2 launches on one CTA instead).
 * fpgm_ci_test_batch: tests[t*(2+d) + 0,1,2..] = x, y, z1..zd; all tests run in one
 * persistent launch.  want_hash != 0 fills table_hash (slower). */
int fpgm_ci_test(fpgm_engine *eng, int32_t x, int32_t y, const int32_t *z, int32_t nz, double alpha,
                 int32_t want_hash, fpgm_ci_result *out);
int fpgm_ci_test_batch(fpgm_engine *eng, const int32_t *tests, int32_t n_tests, int32_t d, double alpha,
                       int32_t want_hash, fpgm_ci_result *out);

/* ---- CI test without allocation ----
 * No counterpart in the reference.  For callers that cannot allocate device memory:
 * their device memory belongs to another allocator (a host framework's caching pool or
 * a fixed arena), or a cudaMalloc is not allowed or would stall the device where they
 * run.  Such a caller already holds its samples on the device; this runs the plain
 * single-test kernel on them and writes one fpgm_ci_result to caller-owned device
 * memory, using only a fixed scratch array of 2^20 + 16,500 ints (about 4.3 MB) inside
 * the library, held by every GPU that loads the library until the process exits.  It
 * calls no cudaMalloc, cudaFree or allocating library routine.
 *   columns  device pointer; variable v at columns + v*pitch, ids already dense
 *            (0 .. states-1, e.g. first-appearance relabelled as fpgm_dataset_upload does);
 *            16-byte aligned, pitch a multiple of 16 and >= n_samples
 *   result   device pointer to one fpgm_ci_result, 8-byte aligned (written when the stream reaches it)
 *   stream   cudaStream_t to run on (NULL: the legacy default stream); the call waits on
 *            it once, to read the tested columns' state counts for the size check
 * Limits: joint table plus marginals of at most 2^20 ints (else FPGM_ERR_UNSUPPORTED),
 * at most 65,536 variables and 255 states per variable.
 * The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) with that device current: make that first call before any
 * stream capture.  The address is kept for the life of the process, so the entry point
 * must not be used on a device after cudaDeviceReset of that device.  All calls share the one scratch array, which keeps the previous
 * call's contents (each call clears what it uses): calls that overlap on the GPU, from
 * other streams or threads, race and must be serialised by the caller. */
int fpgm_ci_test_noalloc(const uint8_t *columns, int64_t pitch, int32_t n_vars, int64_t n_samples, int32_t x,
                         int32_t y, const int32_t *z, int32_t nz, double alpha, int32_t want_hash,
                         fpgm_ci_result *result, void *stream);

/* ---- PC-stable skeleton ----
 * depth follows PCStable(Network*, alpha, depth=1000): levels d = 0 .. depth-1.
 * mode: FPGM_MODE_BATCHED (device-resident level engine) or FPGM_MODE_PLAIN
 * (the reference's control flow on the host, one fpgm_ci_test per CI test).
 * The result stays in the engine until the next call; fetch it below. */
int fpgm_pc_skeleton(fpgm_engine *eng, double alpha, int32_t depth, int32_t mode, fpgm_pc_stats *stats);
int fpgm_pc_result_sizes(fpgm_engine *eng, int32_t *n_nodes, int32_t *n_removed, int64_t *n_sep_vars);
/* adj: n*n bytes (1 = edge kept).  removed: 2*n_removed (a < b pairs, ascending).
 * sep_offsets: n_removed+1.  sep_vars: n_sep_vars (each set ascending, like set<int>). */
int fpgm_pc_result_fetch(fpgm_engine *eng, uint8_t *adj, int32_t *removed, int32_t *sep_offsets,
                         int32_t *sep_vars);

/* ---- orientation (host) ----
 * Reproduces the reference's order-dependent v-structure and Meek-rule pass on
 * a skeleton.  Output edges in the reference's final vec_edges order:
 * out_edges[3*i] = a, [3*i+1] = b, [3*i+2] = 1 for a -> b, 0 for a -- b.
 * out_edges needs room for 3 * (#skeleton edges). */
int fpgm_orient_cpdag(int32_t n, const uint8_t *adj, int32_t n_removed, const int32_t *removed,
                      const int32_t *sep_offsets, const int32_t *sep_vars, int32_t *out_edges,
                      int32_t *out_n_edges);
/* Writes the reference's _struct text (StructureLearning.cpp:238-292) for the edge records
 * fpgm_orient_cpdag produced.  names may be NULL (then "<i>").  num_edges_header is the skeleton
 * edge count the reference prints in the header and iterates over. */
int fpgm_write_struct(const char *path, int32_t n, const char *const *names, const int32_t *edges,
                      int32_t n_edges, int32_t num_edges_header);

/* ---- drop-in job ---- */
int fpgm_bnsl_pcstable(int32_t verbose, int32_t n_threads, int32_t group_size, double alpha,
                       const char *ref_net, const char *train_set, int32_t save_struct);
/* BNL_PCStable (fastpgm_api.cpp:46-75, the command line's -j 1 -m 0): as fpgm_bnsl_pcstable,
 * then maximum-likelihood parameters (Laplace alpha 1) for the learned graph's arcs, written to
 * train_set + "_param" when save_param (ParameterLearning::SaveBNParameter's format). */
int fpgm_bnl_pcstable(int32_t verbose, int32_t n_threads, int32_t group_size, double alpha, const char *ref_net,
                      const char *train_set, int32_t save_struct, int32_t save_param);

/* ---- seeded synthetic data ---- */
int fpgm_generate_network(const fpgm_gen_spec *spec, uint8_t *out_columns, uint8_t *out_card,
                          int32_t *out_parents);
int fpgm_write_csv(const char *path, const uint8_t *columns, int32_t n_vars, int64_t n_samples,
                   const char *name_prefix);

#ifdef __cplusplus
}
#endif

#endif
