// Context, memory, timing and error plumbing of libkvft.
#include "kvft_internal.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <new>

int kv_fail(kvft_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int kv_cuda(kvft_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    int code = (e == cudaErrorMemoryAllocation) ? KVFT_ENOMEM : KVFT_EDEVICE;
    return kv_fail(ctx, code, m);
}

void kv_pack_cache_clear(kvft_ctx *ctx) {
    for (auto &kv : ctx->pack_cache) cudaFree(kv.second.first);
    ctx->pack_cache.clear();
    ctx->scratch_gen++;
}

int kv_launch_check(kvft_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return kv_cuda(ctx, e, what);
    return KVFT_OK;
}

int kv_scratch(kvft_ctx *ctx, const char *key, size_t bytes, void **p) {
    auto it = ctx->scratch.find(key);
    if (it != ctx->scratch.end() && it->second.second >= bytes) {
        *p = it->second.first;
        return KVFT_OK;
    }
    if (ctx->dry) {
        // host memory, every double NaN: a read before any write shows
        if (it != ctx->scratch.end()) {
            std::free(it->second.first);
            ctx->scratch.erase(it);
        }
        size_t b = bytes ? bytes : 256;
        void *q = std::malloc(b);
        if (!q) return kv_fail(ctx, KVFT_ENOMEM, "dry run: host scratch");
        std::memset(q, 0xff, b);
        ctx->scratch[key] = {q, b};
        *p = q;
        return KVFT_OK;
    }
    ctx->scratch_gen++;
    if (it != ctx->scratch.end()) {
        KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(it->second.first);
        ctx->scratch.erase(it);
    }
    void *q = nullptr;
    size_t b = bytes ? bytes : 256;
    KV_CHECK(ctx, cudaMalloc(&q, b));
    ctx->scratch[key] = {q, b};
    *p = q;
    return KVFT_OK;
}

extern "C" {

const char *kvft_status_string(int s) {
    switch (s) {
    case KVFT_OK: return "ok";
    case KVFT_EINVAL: return "invalid argument";
    case KVFT_ENOMEM: return "device memory exhausted";
    case KVFT_EDIVERGE: return "iteration diverged";
    case KVFT_ETIMEOUT: return "device wait timed out";
    case KVFT_EDEVICE: return "CUDA error";
    case KVFT_ENOTCONV: return "not converged";
    default: return "unknown status";
    }
}

int kvft_ctx_create(int device, void *stream, kvft_ctx **out) {
    if (!out) return KVFT_EINVAL;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return KVFT_EDEVICE;
    if (device < 0 || device >= ndev) return KVFT_EINVAL;
    kvft_ctx *c = new (std::nothrow) kvft_ctx();
    if (!c) return KVFT_ENOMEM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return KVFT_EDEVICE; }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return KVFT_EDEVICE;
        }
        c->own_stream = true;
    }
    for (int i = 0; i < 64; i++) cudaEventCreate(&c->ev[i]);
    if (cudaMalloc(&c->dflag, 64 * sizeof(int)) != cudaSuccess) {
        delete c;
        return KVFT_ENOMEM;
    }
    cudaMemsetAsync(c->dflag, 0, 64 * sizeof(int), c->stream);
    *out = c;
    return KVFT_OK;
}

int kvft_ctx_destroy(kvft_ctx *c) {
    if (!c) return KVFT_OK;
    if (c->dry) {
        for (auto &kv : c->scratch) std::free(kv.second.first);
        delete c->dry;
        delete c;
        return KVFT_OK;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto &kv : c->scratch) cudaFree(kv.second.first);
    kv_pack_cache_clear(c);
    if (c->prof) {
        for (auto e : c->prof->pool) cudaEventDestroy(e);
        delete c->prof;
    }
    if (c->l2buf) cudaFree(c->l2buf);
    if (c->dflag) cudaFree(c->dflag);
    if (c->hstage) cudaFreeHost(c->hstage);
    for (int i = 0; i < 64; i++) cudaEventDestroy(c->ev[i]);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return KVFT_OK;
}

const char *kvft_last_error(const kvft_ctx *c) { return c ? c->err.c_str() : "null context"; }

int kvft_dryrun_create(int precision, int digits, kvft_ctx **out) {
    if (!out) return KVFT_EINVAL;
    *out = nullptr;
    kvft_ctx *c = new (std::nothrow) kvft_ctx();
    if (!c) return KVFT_ENOMEM;
    c->dry = new (std::nothrow) std::vector<KvDryOp>();
    if (!c->dry) {
        delete c;
        return KVFT_ENOMEM;
    }
    c->sm_count = 152;
    c->precision = precision;
    c->digits = digits;
    *out = c;
    return KVFT_OK;
}

int kvft_dryrun_count(const kvft_ctx *c, int *count) {
    if (!c || !c->dry || !count) return KVFT_EINVAL;
    *count = (int)c->dry->size();
    return KVFT_OK;
}

int kvft_dryrun_scratch(const kvft_ctx *c, int i, const void **ptr, size_t *bytes) {
    if (!c || !c->dry || !ptr || !bytes || i < 0 || i >= (int)c->scratch.size())
        return KVFT_EINVAL;
    auto it = c->scratch.begin();
    std::advance(it, i);
    *ptr = it->second.first;
    *bytes = it->second.second;
    return KVFT_OK;
}

int kvft_dryrun_op(const kvft_ctx *c, int i, int *ints, long long *longs, double *dbls,
                   const void **ptrs) {
    if (!c || !c->dry || i < 0 || i >= (int)c->dry->size() || !ints || !longs || !dbls ||
        !ptrs)
        return KVFT_EINVAL;
    const KvDryOp &op = (*c->dry)[i];
    // ints: kind M N K batch | A.r A.c B.r B.c C.r C.c sizes (18) | dims (4) | ng rank
    //       full nv no (5) = 32
    // longs: A.r A.c B.r B.c C.r C.c strides (18) | A.bst B.bst C.bst | ss (4) ds (4)
    //        sbst dbst | P = 32
    const KIdx *ix[6] = {&op.A.r, &op.A.c, &op.B.r, &op.B.c, &op.C.r, &op.C.c};
    ints[0] = op.kind, ints[1] = op.M, ints[2] = op.N, ints[3] = op.K, ints[4] = op.batch;
    for (int k = 0; k < 6; k++)
        for (int d = 0; d < 3; d++) {
            ints[5 + 3 * k + d] = ix[k]->size[d];
            longs[3 * k + d] = ix[k]->st[d];
        }
    for (int d = 0; d < 4; d++) {
        ints[23 + d] = op.dims[d];
        longs[21 + d] = op.ss[d];
        longs[25 + d] = op.ds[d];
    }
    ints[27] = op.ng, ints[28] = op.rank, ints[29] = op.full, ints[30] = op.nv,
    ints[31] = op.no;
    longs[18] = op.A.bst, longs[19] = op.B.bst, longs[20] = op.C.bst;
    longs[29] = op.sbst, longs[30] = op.dbst, longs[31] = op.P;
    dbls[0] = op.alpha, dbls[1] = op.beta;
    const void *p[11] = {op.A.p, op.B.p, op.C.p, op.src, op.dst, op.ti,
                         op.G,   op.ev,  op.eo,  op.src2, op.res};
    for (int k = 0; k < 11; k++) ptrs[k] = p[k];
    return KVFT_OK;
}

int kvft_set_precision(kvft_ctx *c, int precision, int digits) {
    if (!c) return KVFT_EINVAL;
    if (precision < KVFT_PREC_FP64 || precision > KVFT_PREC_MIXED)
        return kv_fail(c, KVFT_EINVAL, "unknown precision");
    if (precision != KVFT_PREC_FP64 && (digits < 2 || digits > 9))
        return kv_fail(c, KVFT_EINVAL, "digit levels must be in [2, 9]");
    c->precision = precision;
    c->digits = digits;
    return KVFT_OK;
}

int kvft_alloc(kvft_ctx *c, size_t bytes, void **p) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_alloc: not on a dry-run context");
    if (!c || !p) return KVFT_EINVAL;
    cudaSetDevice(c->device);
    KV_CHECK(c, cudaMalloc(p, bytes ? bytes : 16));
    return KVFT_OK;
}

int kvft_free(kvft_ctx *c, void *p) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_free: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    KV_CHECK(c, cudaStreamSynchronize(c->stream));
    KV_CHECK(c, cudaFree(p));
    return KVFT_OK;
}

int kvft_h2d(kvft_ctx *c, void *dst, const void *src, size_t bytes) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_h2d: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    KV_CHECK(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return KVFT_OK;
}

int kvft_d2h(kvft_ctx *c, void *dst, const void *src, size_t bytes) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_d2h: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    KV_CHECK(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    KV_CHECK(c, cudaStreamSynchronize(c->stream));
    return KVFT_OK;
}

int kvft_memset(kvft_ctx *c, void *p, int v, size_t bytes) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_memset: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    KV_CHECK(c, cudaMemsetAsync(p, v, bytes, c->stream));
    return KVFT_OK;
}

int kvft_sync(kvft_ctx *c) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_sync: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    KV_CHECK(c, cudaStreamSynchronize(c->stream));
    return KVFT_OK;
}

int kvft_event_record(kvft_ctx *c, int slot) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_event_record: not on a dry-run context");
    if (!c || slot < 0 || slot >= 64) return KVFT_EINVAL;
    KV_CHECK(c, cudaEventRecord(c->ev[slot], c->stream));
    return KVFT_OK;
}

int kvft_event_elapsed_ms(kvft_ctx *c, int s0, int s1, float *ms) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_event_elapsed_ms: not on a dry-run context");
    if (!c || s0 < 0 || s0 >= 64 || s1 < 0 || s1 >= 64 || !ms) return KVFT_EINVAL;
    KV_CHECK(c, cudaEventSynchronize(c->ev[s1]));
    KV_CHECK(c, cudaEventElapsedTime(ms, c->ev[s0], c->ev[s1]));
    return KVFT_OK;
}

int kvft_launch_count(kvft_ctx *c, uint64_t *count) {
    if (!c || !count) return KVFT_EINVAL;
    *count = c->launches;
    return KVFT_OK;
}

}  // extern "C"

// ---- live launch timing ------------------------------------------------------
int kv_prof_mark(kvft_ctx *ctx, size_t *slot) {
    KvProf *p = ctx->prof;
    if (p->used == p->pool.size()) {
        cudaEvent_t e;
        KV_CHECK(ctx, cudaEventCreate(&e));
        p->pool.push_back(e);
    }
    *slot = p->used++;
    KV_CHECK(ctx, cudaEventRecord(p->pool[*slot], ctx->stream));
    return KVFT_OK;
}

void kv_prof_add(kvft_ctx *ctx, int cat, size_t e0, size_t e1, double work) {
    KvProf::Rec r{cat, e0, e1, work, {0, 0, 0, 0}};
    if (cat == KV_CAT_GEMM6 || cat == KV_CAT_GEMM || cat == KV_CAT_PACK)
        for (int k = 0; k < 4; k++) r.shape[k] = ctx->prof->shape[k];
    ctx->prof->recs.push_back(r);
}

KvProfScope::KvProfScope(kvft_ctx *c, int k, double w)
    : ctx(c), cat(k), work(w), e0(0), on(c->prof && c->prof->on) {
    if (on && kv_prof_mark(ctx, &e0) != KVFT_OK) on = false;
}

KvProfScope::~KvProfScope() {
    size_t e1;
    if (on && kv_prof_mark(ctx, &e1) == KVFT_OK) kv_prof_add(ctx, cat, e0, e1, work);
}

extern "C" int kvft_profile_begin(kvft_ctx *c) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_profile_begin: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    if (!c->prof) c->prof = new KvProf();
    c->prof->on = true;
    c->prof->used = 0;
    c->prof->recs.clear();
    return KVFT_OK;
}

extern "C" int kvft_profile_records(kvft_ctx *c, int max, int *count, int *cat, float *ms,
                                    double *work) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_profile_records: not on a dry-run context");
    if (!c || !c->prof || !count || max < 0 || (max > 0 && (!cat || !ms || !work)))
        return KVFT_EINVAL;
    KV_CHECK(c, cudaStreamSynchronize(c->stream));
    const auto &recs = c->prof->recs;
    *count = (int)recs.size();
    for (int i = 0; i < max && i < (int)recs.size(); i++) {
        float t = 0.f;
        KV_CHECK(c, cudaEventElapsedTime(&t, c->prof->pool[recs[i].e0], c->prof->pool[recs[i].e1]));
        cat[i] = recs[i].cat;
        ms[i] = t;
        work[i] = recs[i].work;
    }
    return KVFT_OK;
}

extern "C" int kvft_profile_shapes(kvft_ctx *c, int max, int *count, int *shapes) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_profile_shapes: not on a dry-run context");
    if (!c || !c->prof || !count || max < 0 || (max > 0 && !shapes)) return KVFT_EINVAL;
    const auto &recs = c->prof->recs;
    *count = (int)recs.size();
    for (int i = 0; i < max && i < (int)recs.size(); i++)
        for (int k = 0; k < 4; k++) shapes[4 * i + k] = recs[i].shape[k];
    return KVFT_OK;
}

extern "C" int kvft_profile_end(kvft_ctx *c, kvft_profile_stats *out) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_profile_end: not on a dry-run context");
    if (!c || !c->prof || !out) return KVFT_EINVAL;
    KV_CHECK(c, cudaStreamSynchronize(c->stream));
    memset(out, 0, sizeof(*out));
    for (auto &r : c->prof->recs) {
        float ms = 0.f;
        KV_CHECK(c, cudaEventElapsedTime(&ms, c->prof->pool[r.e0], c->prof->pool[r.e1]));
        out->launches[r.cat] += 1;
        out->ms[r.cat] += ms;
        out->work[r.cat] += r.work;
    }
    c->prof->on = false;
    c->prof->recs.clear();
    c->prof->used = 0;
    return KVFT_OK;
}

__global__ void kv_flush_kernel(uint4 *p, size_t n, unsigned salt) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) p[i] = make_uint4(salt, (unsigned)i, salt, 0u);
}

extern "C" int kvft_flush_l2(kvft_ctx *c) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_flush_l2: not on a dry-run context");
    if (!c) return KVFT_EINVAL;
    const size_t bytes = 256ull << 20;  // twice the 129 MB L2
    if (!c->l2buf) KV_CHECK(c, cudaMalloc(&c->l2buf, bytes));
    static unsigned salt = 1;
    kv_flush_kernel<<<c->sm_count * 4, 512, 0, c->stream>>>((uint4 *)c->l2buf, bytes / 16, salt++);
    return kv_launch_check(c, "flush_l2");
}

extern "C" int kvft_mem_info(kvft_ctx *c, size_t *free_bytes, size_t *total_bytes) {
    if (c && c->dry) return kv_fail(c, KVFT_EINVAL, "kvft_mem_info: not on a dry-run context");
    if (!c || !free_bytes || !total_bytes) return kv_fail(c, KVFT_EINVAL, "kvft_mem_info: bad argument");
    cudaSetDevice(c->device);
    KV_CHECK(c, cudaMemGetInfo(free_bytes, total_bytes));
    return KVFT_OK;
}

extern "C" int kvft_set_workspace_limit(kvft_ctx *c, size_t bytes) {
    if (!c) return KVFT_EINVAL;
    c->workspace_limit = bytes;
    return KVFT_OK;
}
