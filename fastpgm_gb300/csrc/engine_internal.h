// Internal helpers shared by the engine's translation units.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace fpgm {
// Records a printf-style message as the calling thread's last error and returns code.
int set_error(int code, const char *fmt, ...);

// Device allocations of the engine go through these: cudaMalloc / cudaFree with a
// process-wide byte count, refused with FPGM_ERR_OOM beyond FPGM_DEVICE_MEM_CAP bytes when
// that is set (the allocation-failure path, testable without exhausting a GPU).
int dev_alloc(void **p, size_t bytes);
void dev_free(void *p, size_t bytes);

#define RET_IF(call)                  \
    do {                              \
        int r_ = (call);              \
        if (r_ != 0) return r_;       \
    } while (0)

// Level-0 pair counts on the tensor cores (gram.cu): the Gram matrix of the samples'
// one-hot matrix holds every pair's joint table.
struct GramLevel0;
GramLevel0 *gram_create();
void gram_destroy(GramLevel0 *g);
// Lays out the one-hot rows of one dataset (n variables, host cardinalities, S samples,
// device columns / byte offsets / cardinalities) and sizes the buffers.  *ok is false when
// the path does not apply (a pair table beyond a warp's shared slice, too many rows).
int gram_plan(GramLevel0 *g, int n, const uint8_t *h_card, int64_t S, const uint8_t *d_cols,
              const int64_t *d_var_off, const uint8_t *d_card, int num_sms, cudaStream_t stream, bool *ok);
// Enqueues the one-hot build and the Gram GEMM; *err is raised if a bounded wait gave up.
int gram_run(GramLevel0 *g, cudaStream_t stream, unsigned long long *err, int *launches);
const int32_t *gram_counts(const GramLevel0 *g);   // G, row pitch gram_ld(g) int32
const int32_t *gram_row_off(const GramLevel0 *g);  // device: first one-hot row of each variable
int gram_ld(const GramLevel0 *g);
int gram_slice_ints(const GramLevel0 *g);          // largest pair table + marginals (ints), 16-aligned
double gram_flops(const GramLevel0 *g);            // tensor-core flops of one gram_run
}  // namespace fpgm
