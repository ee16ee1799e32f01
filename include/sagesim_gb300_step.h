/*
 * sagesim_gb300_step.h -- device-side API for step functions compiled with
 * sg_compile_step (NVRTC). The engine prepends this header to the step source;
 * a step is
 *
 *     __device__ void my_step(const sg_ctx &ctx, int i) { ... }
 *
 * and runs once per agent i of its range per tick, like a SAGESim step
 * function (sagesim/model.py:2312-2353 calls it per agent index). Reads
 * (ctx.i32 / ctx.f32) of double-buffered properties see tick-start values;
 * writes (ctx.set_i32 / ctx.set_f32) go to the write buffer, the reference's
 * write_* redirection (sagesim/model.py:2142-2220). Properties added with
 * double_buffered = 0 are read and written in place (no_double_buffer,
 * sagesim/breed.py:68-99). ctx.rand_uniform(i, salt) is SAGESim's
 * rand_uniform_philox(tick, agent_index, salt) with the seed and the agent's
 * logical id filled in, as the reference's _inject_seed rewrite does
 * (sagesim/model.py:1903-1953).
 */
#ifndef SAGESIM_GB300_STEP_H
#define SAGESIM_GB300_STEP_H

/* Per-property device view: two buffers, which one is read at relative tick r
 * is (cur0 + r) & 1 for a double-buffered property, buffer 0 otherwise. rows is
 * the agent count, or the row count of a breed-local array. */
typedef struct sg_prop_dev {
    void *buf0;
    void *buf1;
    int width;
    int dbuf;
    int cur0;
    int dtype;
    long long rows;
} sg_prop_dev;

/* Kernel parameter of a compiled step (identical layout on host and device). */
typedef struct sg_step_args {
    const int *tiles;        /* [ntiles][4]: seg, begin, end, pad               */
    int ntiles;
    int r;                   /* tick relative to the run start                  */
    long long tick0;         /* absolute tick at r == 0                         */
    unsigned int key;        /* seed mod 2^32                                   */
    int nprops;
    const unsigned int *lids; /* RNG key (lid mod 2^32) per agent, NULL = index  */
    const int *off;          /* CSR offsets                                     */
    const int *idx;          /* CSR indices                                     */
    const double *g;         /* globals                                         */
    const sg_prop_dev *props;
    long long n;             /* agent count                                     */
} sg_step_args;

#ifdef __CUDACC__
struct sg_ctx {
    long long tick;
    unsigned int key;
    unsigned int c0b;
    int r;
    const unsigned int *lids;
    const int *off;
    const int *idx;
    const double *g;
    const sg_prop_dev *props;

    __device__ __forceinline__ const void *rd(int p) const
    {
        const sg_prop_dev &d = props[p];
        return (d.dbuf && ((d.cur0 + r) & 1)) ? d.buf1 : d.buf0;
    }
    __device__ __forceinline__ void *wr(int p) const
    {
        const sg_prop_dev &d = props[p];
        if (!d.dbuf) return d.buf0;
        return ((d.cur0 + r) & 1) ? d.buf0 : d.buf1;
    }
    __device__ __forceinline__ int width(int p) const { return props[p].width; }
    __device__ __forceinline__ int i32(int p, int i, int c = 0) const
    {
        return ((const int *)rd(p))[(long long)i * props[p].width + c];
    }
    __device__ __forceinline__ float f32(int p, int i, int c = 0) const
    {
        return ((const float *)rd(p))[(long long)i * props[p].width + c];
    }
    __device__ __forceinline__ void set_i32(int p, int i, int v, int c = 0) const
    {
        ((int *)wr(p))[(long long)i * props[p].width + c] = v;
    }
    __device__ __forceinline__ void set_f32(int p, int i, float v, int c = 0) const
    {
        ((float *)wr(p))[(long long)i * props[p].width + c] = v;
    }
    /* Breed-local arrays (sagesim/model.py:620-650): element (row, c) of the
     * row-major [rows][width] float32 array p, row from the array's index map
     * (ctx.i32(p_idx, agent), -1 for agents of other breeds). A row or column
     * outside the array reads 0 and drops the write. */
    __device__ __forceinline__ bool in_array(int p, long long row, long long c) const
    {
        return (unsigned long long)row < (unsigned long long)props[p].rows &&
               (unsigned long long)c < (unsigned long long)props[p].width;
    }
    __device__ __forceinline__ float arr_f32(int p, long long row, long long c) const
    {
        return in_array(p, row, c) ? ((const float *)rd(p))[row * props[p].width + c] : 0.0f;
    }
    __device__ __forceinline__ void set_arr_f32(int p, long long row, float v, long long c) const
    {
        if (in_array(p, row, c)) ((float *)wr(p))[row * props[p].width + c] = v;
    }
    /* CSR rows: sagesim/utils.py:36-57 (get_num_neighbors / get_neighbor). */
    __device__ __forceinline__ int degree(int i) const { return off[i + 1] - off[i]; }
    __device__ __forceinline__ int neighbor(int i, int k) const { return idx[off[i] + k]; }
    __device__ __forceinline__ unsigned int lid(int i) const
    {
        return lids ? lids[i] : (unsigned int)i;
    }
    /* sagesim/math_utils.py:106-189 */
    __device__ __forceinline__ double rand_uniform(int i, long long salt) const
    {
        return (double)sg_philox_k23(c0b + (unsigned int)(unsigned long long)salt, lid(i), key) /
               8388608.0;
    }
    /* sagesim/math_utils.py:231-255 */
    __device__ __forceinline__ double rand_normal(int i, long long salt) const
    {
        const double u1 = rand_uniform(i, salt);
        const double u2 = rand_uniform(i, salt + 73856093LL);
        return __dmul_rn(sqrt(__dmul_rn(-2.0, log(__dadd_rn(u1, 1e-10)))),
                         cos(__dmul_rn(6.283185307179586, u2)));
    }
};
#endif /* __CUDACC__ */

#endif /* SAGESIM_GB300_STEP_H */
