// Serving loop: continuous batching of image / likelihood requests.
//
// The reference simulates one ImageModel.image call per XLA program
// (image_model.py:432-492), or a jax.vmap over a fixed batch.  A server here
// owns one worker thread that
//   * releases submitted requests into per-bucket FIFO queues once their
//     release time has passed (a bucket = one compiled model: profile lists,
//     grid, supersampling, PSF size, precision and noise options; with
//     mixed_grids, image requests of every grid and PSF size (mixed_grids = 2:
//     and supersampling factor) of one profile stack and precision share a
//     bucket, whose batches run through lensgb_image_mixed);
//   * keeps up to n_streams batches in flight, one per CUDA stream, each batch
//     a single lensgb_image / lensgb_loglike launch sequence over up to
//     max_batch requests of one bucket -- requests that arrive while others
//     are on the GPU join the next batch as soon as a stream frees up;
//   * stages each request's parameters, PSF, data, noise map and mask into
//     device buffers of an execution context (grow-only, per bucket), whose
//     total size is held under hbm_budget_bytes: idle contexts are evicted
//     (least recently used first) to admit new ones, and requests wait in
//     their queue while the budget is exhausted by batches in flight;
//   * optionally replays a CUDA graph captured for a context and batch size
//     after its first eager run.
// Each batch is one sequence of stream operations on buffers the context owns
// -- copies of the pinned staging, gather kernels that read page-locked
// request inputs through a pointer table, the image kernels, and a scatter
// kernel that writes every image straight into its request's page-locked
// host buffer (pageable buffers get a pinned staging copy, finished by the
// worker) -- so a replayed graph needs only freshly staged inputs.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "launch.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    lensgb_request r;
    long long ticket = 0;
    int bucket = -1;
    std::atomic<int> state{LENSGB_REQ_QUEUED};
    int rc = LENSGB_OK;
    bool out_pinned = false;  // image_out is device-readable (page-locked host or device
                              // memory): the device writes it directly
    int in_pinned = 0;        // bits 0..2: data / noise_map / mask, bit 4: psf are
                              // device-readable, read in place by the gather kernels
    long long npix = 0;       // ny x nx of the request's grid
    int k2 = 0;               // PSF elements of the request
    long long t_submit = 0, t_release = 0, t_admit = 0, t_done = 0;
};

struct BucketKey {
    lensgb_model_desc desc;
    int likelihood;      // 0: image only; 1: image + logL
    int has_noise, has_mask;
    double background_rms, exposure_time;
    int psf_on_device;   // PSFs in device memory: exact-model buckets gather them in place
    bool operator<(const BucketKey& o) const {
        int c = memcmp(&desc, &o.desc, sizeof desc);
        if (c) return c < 0;
        if (psf_on_device != o.psf_on_device) return psf_on_device < o.psf_on_device;
        if (likelihood != o.likelihood) return likelihood < o.likelihood;
        if (has_noise != o.has_noise) return has_noise < o.has_noise;
        if (has_mask != o.has_mask) return has_mask < o.has_mask;
        if (background_rms != o.background_rms) return background_rms < o.background_rms;
        return exposure_time < o.exposure_time;
    }
};

// Pointer-table planes of a context: image outputs, data, noise map, mask, PSF.
constexpr int PTR_PLANES = 5, PSF_PLANE = 4;

struct Context {
    int bucket = -1;
    lensgb_model* model = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    int cap = 0;             // batch capacity of the buffers below (requests)
    long long pix_cap = 0;   // image pixels and PSF elements the buffers hold
    long long kel_cap = 0;
    size_t bytes = 0;        // device bytes held (buffers + model scratch)
    double* rows_dev = nullptr;
    void* psf_dev = nullptr;
    void* img_dev = nullptr;
    double* data_dev = nullptr;
    double* noise_dev = nullptr;
    double* mask_dev = nullptr;
    double* logl_dev = nullptr;
    double* rows_host = nullptr;  // pinned staging
    unsigned char* psf_host = nullptr;
    double* logl_host = nullptr;
    unsigned char* img_host = nullptr;  // pinned staging for pageable caller buffers
    unsigned char* in_host = nullptr;   // pinned staging of pageable data / noise / mask
    void** ptr_host = nullptr;          // pinned pointer tables: out[cap], data, noise, mask,
    void** ptr_dev = nullptr;           // psf, then (mixed buckets) cap + 1 image byte offsets
    long long* boff_host = nullptr;     // the byte-offset part of ptr_host / ptr_dev
    long long* boff_dev = nullptr;
    // mixed buckets: one page-locked staging block -- rows | PSFs | output
    // pointers + byte offsets | mixed-launch tables -- and its device mirror,
    // refreshed by one copy of fixed size (rows_host ... point into it)
    unsigned char* stage_host = nullptr;
    unsigned char* stage_dev = nullptr;
    size_t stage_bytes = 0, o_tab = 0;
    lensgb::MixedLayout ml;
    std::vector<lensgb_system_grid> grids;  // the batch's grids
    lensgb::MixedGrid mgrid;                // the batch's launch shape
    bool busy = false;
    long long last_used = 0;
    std::vector<Req*> batch;
    // uniform buckets: batch size -> graph; mixed buckets: launch shape -> graph
    std::map<long long, cudaGraphExec_t> graphs;
    std::map<long long, int> eager_runs;    // eager launches so far, same keys
};

struct Bucket {
    BucketKey key;
    bool mixed = false;  // requests of different grids / PSF sizes (lensgb_image_mixed)
    int n_params = 0;
    long long npix = 0;  // uniform buckets: pixels and PSF elements per request
    int k2 = 0;
    size_t esz = 4;      // image element size
    std::deque<Req*> queue;
    std::vector<Context*> ctx;
};

}  // namespace

struct lensgb_server {
    lensgb_server_config cfg;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    int device = 0;
    int n_sms = 1;                            // SMs of the device (launch shapes), read at create
    std::deque<Req> reqs;                     // stable storage, index = ticket
    std::vector<Req*> incoming;               // submitted, not yet released
    std::vector<Bucket*> buckets;             // guarded by mu (appended by submit)
    std::map<BucketKey, int> bucket_index;    // exact request key -> bucket
    std::map<BucketKey, int> mixed_index;     // grid-free key -> mixed bucket
    std::vector<Bucket*> wb;                  // the worker's copy of `buckets`
    std::vector<Context*> contexts;
    std::vector<long long> pre_pix, pre_kel;  // worker scratch: prefix sums of a queue head
    size_t bytes_held = 0;
    size_t peak_bytes = 0;
    int inflight = 0;
    std::atomic<long long> n_done{0};
    lensgb_server_stats stats;
    std::atomic<bool> stop{false};
    std::thread worker;

    long long now() const {
        return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
    }
};

namespace {

int serr(int code, const std::string& m) {
    lensgb::set_last_error(m);
    return code;
}

// What a batch needs: requests, image pixels, PSF elements.
struct Need {
    int n;
    long long pix, kel;
};

size_t context_bytes(const Bucket& b, const Need& d) {
    // buffers owned by the context
    size_t bytes = (size_t)d.n * ((size_t)b.n_params * 8 + 8) + (size_t)d.kel * b.esz +
                   (size_t)d.pix * b.esz;
    if (b.key.likelihood) {
        bytes += (size_t)d.pix * 8;
        if (b.key.has_noise) bytes += (size_t)d.pix * 8;
        if (b.key.has_mask) bytes += (size_t)d.pix * 8;
    }
    // model scratch: records, coefficient tables, un-convolved image, refine list
    const lensgb_model_desc& m = b.key.desc;
    const size_t nprof = (size_t)(m.n_lens + m.n_source + m.n_lens_light);
    bytes += (size_t)d.n * (nprof * (32 * 8 + 36 * 4) + (size_t)m.n_lens * 500 * 12) +
             (size_t)d.pix * (b.esz + 4);
    // mixed launches: ray and convolution CTA tables, per-system grids
    if (b.mixed) bytes += (size_t)d.pix / 16 + (size_t)d.n * 160 + 4096;
    return bytes;
}

void free_context_buffers(Context* c) {
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
    c->graphs.clear();
    c->eager_runs.clear();
    if (c->stage_host) {
        // the staging buffers are parts of one block
        cudaFreeHost(c->stage_host);
        cudaFree(c->stage_dev);
        c->stage_host = c->stage_dev = nullptr;
        c->stage_bytes = 0;
        c->rows_dev = nullptr;
        c->psf_dev = nullptr;
        c->ptr_dev = nullptr;
        c->rows_host = nullptr;
        c->psf_host = nullptr;
        c->ptr_host = nullptr;
    }
    cudaFree(c->rows_dev);
    cudaFree(c->psf_dev);
    cudaFree(c->img_dev);
    cudaFree(c->data_dev);
    cudaFree(c->noise_dev);
    cudaFree(c->mask_dev);
    cudaFree(c->logl_dev);
    cudaFreeHost(c->rows_host);
    cudaFreeHost(c->psf_host);
    cudaFreeHost(c->logl_host);
    cudaFreeHost(c->img_host);
    cudaFreeHost(c->in_host);
    cudaFreeHost(c->ptr_host);
    cudaFree(c->ptr_dev);
    c->img_host = nullptr;
    c->in_host = nullptr;
    c->ptr_host = nullptr;
    c->ptr_dev = nullptr;
    c->boff_host = c->boff_dev = nullptr;
    c->rows_dev = nullptr;
    c->psf_dev = c->img_dev = nullptr;
    c->data_dev = c->noise_dev = c->mask_dev = c->logl_dev = nullptr;
    c->rows_host = nullptr;
    c->psf_host = nullptr;
    c->logl_host = nullptr;
    c->cap = 0;
    c->pix_cap = c->kel_cap = 0;
}

void destroy_context(lensgb_server* s, Context* c) {
    free_context_buffers(c);
    if (c->model) lensgb_model_destroy(c->model);
    if (c->done) cudaEventDestroy(c->done);
    if (c->stream) cudaStreamDestroy(c->stream);
    s->bytes_held -= c->bytes;
    delete c;
}

// Evict idle contexts (least recently used first) until `need` more bytes fit.
bool make_room(lensgb_server* s, size_t need, const Context* keep) {
    while (s->bytes_held + need > (size_t)s->cfg.hbm_budget_bytes) {
        Context* victim = nullptr;
        for (Context* c : s->contexts)
            if (!c->busy && c != keep && (!victim || c->last_used < victim->last_used)) victim = c;
        if (!victim) return false;
        Bucket& b = *s->wb[victim->bucket];
        b.ctx.erase(std::find(b.ctx.begin(), b.ctx.end(), victim));
        s->contexts.erase(std::find(s->contexts.begin(), s->contexts.end(), victim));
        destroy_context(s, victim);
        s->stats.evictions++;
    }
    return true;
}

// Grow a context to hold a batch of `d` (capacities double; requests up to
// max_batch).
int grow_context(lensgb_server* s, Context* c, const Need& d) {
    if (d.n <= c->cap && d.pix <= c->pix_cap && d.kel <= c->kel_cap) return LENSGB_OK;
    Bucket& b = *s->wb[c->bucket];
    int cap = c->cap > 0 ? c->cap : 1;
    while (cap < d.n) cap *= 2;
    if (cap > s->cfg.max_batch) cap = s->cfg.max_batch;
    long long pix_cap, kel_cap;
    if (b.mixed) {
        pix_cap = std::max<long long>(c->pix_cap, 4096);
        while (pix_cap < d.pix) pix_cap *= 2;
        kel_cap = std::max<long long>(c->kel_cap, 256);
        while (kel_cap < d.kel) kel_cap *= 2;
    } else {
        pix_cap = (long long)cap * b.npix;
        kel_cap = (long long)cap * b.k2;
    }
    const Need nd{cap, pix_cap, kel_cap};
    const size_t nb = context_bytes(b, nd);
    if (nb > c->bytes && !make_room(s, nb - c->bytes, c)) return LENSGB_ERR_OOM;
    free_context_buffers(c);
    s->bytes_held -= c->bytes;
    c->bytes = 0;
    const size_t P = (size_t)b.n_params, np = (size_t)pix_cap, nk = (size_t)kel_cap;
    const size_t ptr_bytes = (size_t)cap * PTR_PLANES * sizeof(void*) + ((size_t)cap + 1) * 8;
    bool ok;
    if (b.mixed) {
        auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
        c->ml = lensgb::mixed_layout(cap);
        const size_t o_psf = al(cap * P * 8 + 8), o_ptr = al(o_psf + nk * b.esz + 16);
        c->o_tab = al(o_ptr + ptr_bytes);
        c->stage_bytes = c->o_tab + c->ml.bytes;
        ok = cudaMallocHost(&c->stage_host, c->stage_bytes) == cudaSuccess &&
             cudaMalloc(&c->stage_dev, c->stage_bytes) == cudaSuccess &&
             cudaMalloc(&c->img_dev, np * b.esz) == cudaSuccess &&
             cudaMalloc(&c->logl_dev, cap * 8) == cudaSuccess &&
             cudaMallocHost(&c->logl_host, cap * 8) == cudaSuccess &&
             cudaMallocHost(&c->img_host, np * b.esz) == cudaSuccess;
        if (ok) {
            memset(c->stage_host, 0, c->stage_bytes);
            c->rows_host = (double*)c->stage_host;
            c->rows_dev = (double*)c->stage_dev;
            c->psf_host = c->stage_host + o_psf;
            c->psf_dev = c->stage_dev + o_psf;
            c->ptr_host = (void**)(c->stage_host + o_ptr);
            c->ptr_dev = (void**)(c->stage_dev + o_ptr);
            ok = lensgb::mixed_reserve(c->model, cap, pix_cap, 256) == LENSGB_OK;
        }
    } else {
        ok = cudaMalloc(&c->rows_dev, cap * P * 8 + 8) == cudaSuccess &&
             cudaMalloc(&c->psf_dev, nk * b.esz + 16) == cudaSuccess &&
             cudaMalloc(&c->img_dev, np * b.esz) == cudaSuccess &&
             cudaMalloc(&c->logl_dev, cap * 8) == cudaSuccess &&
             cudaMallocHost(&c->rows_host, cap * P * 8 + 8) == cudaSuccess &&
             cudaMallocHost(&c->psf_host, nk * b.esz + 16) == cudaSuccess &&
             cudaMallocHost(&c->logl_host, cap * 8) == cudaSuccess &&
             cudaMallocHost(&c->img_host, np * b.esz) == cudaSuccess &&
             cudaMallocHost(&c->ptr_host, ptr_bytes) == cudaSuccess &&
             cudaMalloc(&c->ptr_dev, ptr_bytes) == cudaSuccess;
    }
    if (ok && b.key.likelihood) {
        ok = cudaMalloc(&c->data_dev, np * 8) == cudaSuccess;
        if (ok && b.key.has_noise) ok = cudaMalloc(&c->noise_dev, np * 8) == cudaSuccess;
        if (ok && b.key.has_mask) ok = cudaMalloc(&c->mask_dev, np * 8) == cudaSuccess;
        const int planes = 1 + b.key.has_noise + b.key.has_mask;
        if (ok) ok = cudaMallocHost(&c->in_host, planes * np * 8) == cudaSuccess;
    }
    if (ok) ok = lensgb_model_reserve(c->model, cap) == LENSGB_OK;
    if (!ok) {
        cudaGetLastError();
        free_context_buffers(c);
        return LENSGB_ERR_OOM;
    }
    c->boff_host = (long long*)(c->ptr_host + (size_t)cap * PTR_PLANES);
    c->boff_dev = (long long*)(c->ptr_dev + (size_t)cap * PTR_PLANES);  // staging block when mixed
    c->cap = cap;
    c->pix_cap = pix_cap;
    c->kel_cap = kel_cap;
    c->bytes = nb;
    s->bytes_held += nb;
    s->peak_bytes = std::max(s->peak_bytes, s->bytes_held);
    return LENSGB_OK;
}

Context* new_context(lensgb_server* s, int bucket) {
    Bucket& b = *s->wb[bucket];
    Context* c = new Context();
    c->bucket = bucket;
    if (lensgb_model_create(&b.key.desc, &c->model) != LENSGB_OK ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (c->model) lensgb_model_destroy(c->model);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return nullptr;
    }
    b.ctx.push_back(c);
    s->contexts.push_back(c);
    return c;
}

// Copies n blocks between a contiguous device array and the per-request
// buffers named by a pointer table (page-locked host memory, which the GPU
// reads and writes directly): block i is `bytes` long at i * bytes, or, with
// byte offsets `boff` (n + 1 entries), boff[i + 1] - boff[i] long at boff[i].
// n_dev (or null): device count of blocks present, <= gridDim.y.
// to_table = 1: device -> table.
__global__ void table_copy_kernel(unsigned char* dev, void* const* table, size_t bytes,
                                  const long long* boff, const int* n_dev, int to_table) {
    const int i = blockIdx.y;
    if (n_dev && i >= *n_dev) return;
    size_t o = (size_t)i * bytes;
    if (boff) {
        o = (size_t)boff[i];
        bytes = (size_t)(boff[i + 1] - boff[i]);
    }
    unsigned char* d = dev + o;
    unsigned char* h = (unsigned char*)table[i];
    const uintptr_t al = ((uintptr_t)d) | ((uintptr_t)h) | (uintptr_t)bytes;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((al & 15) == 0) {
        uint4* dv = (uint4*)d;
        uint4* hv = (uint4*)h;
        for (size_t j = k; j < bytes / 16; j += stride) {
            if (to_table)
                hv[j] = dv[j];
            else
                dv[j] = hv[j];
        }
    } else if ((al & 3) == 0) {
        unsigned* dw = (unsigned*)d;
        unsigned* hw = (unsigned*)h;
        for (size_t j = k; j < bytes / 4; j += stride) {
            if (to_table)
                hw[j] = dw[j];
            else
                dw[j] = hw[j];
        }
    } else {
        for (size_t j = k; j < bytes; j += stride) {
            if (to_table)
                h[j] = d[j];
            else
                d[j] = h[j];
        }
    }
}

// `bytes`: the block size, or with boff the largest block (sizes the grid).
void table_copy(unsigned char* dev, void* const* table, size_t bytes, int n, int to_table,
                cudaStream_t st, const long long* boff = nullptr, const int* n_dev = nullptr) {
    const size_t units = (bytes % 16 == 0) ? bytes / 16 : (bytes % 4 == 0 ? bytes / 4 : bytes);
    unsigned bx = (unsigned)std::min<size_t>((units + 255) / 256, 64);
    dim3 grid(bx > 0 ? bx : 1, (unsigned)n);
    table_copy_kernel<<<grid, 256, 0, st>>>(dev, table, bytes, boff, n_dev, to_table);
}

// Launch sequence of one batch on the context's stream.  Graph-capturable:
// stream operations only, on buffers owned by the context (pinned staging,
// pointer tables, device arrays), so a replay needs only fresh staging.
int launch_batch(lensgb_server* s, Context* c, int n) {
    Bucket& b = *s->wb[c->bucket];
    cudaStream_t st = c->stream;
    const size_t P = (size_t)b.n_params;
    if (b.mixed) {
        // systems of different grids: the whole staging block in one copy, the
        // mixed launch (system count read on the device), then every image to
        // its request's host buffer
        const lensgb::MixedGrid& gr = c->mgrid;
        if (cudaMemcpyAsync(c->stage_dev, c->stage_host, c->stage_bytes, cudaMemcpyHostToDevice,
                            st) != cudaSuccess)
            return LENSGB_ERR_CUDA;
        const unsigned char* tab = c->stage_dev + c->o_tab;
        int rc = lensgb::mixed_launch(c->model, c->rows_dev, c->cap, tab, c->ml, gr, c->psf_dev,
                                      c->img_dev, 0, st);
        if (rc) return rc;
        table_copy((unsigned char*)c->img_dev, c->ptr_dev, (size_t)16 * 256 * 16, c->cap, 1, st,
                   c->boff_dev, (const int*)(tab + c->ml.o_n));
        return cudaGetLastError() == cudaSuccess ? LENSGB_OK : LENSGB_ERR_CUDA;
    }
    const int planes = b.key.likelihood ? 1 + b.key.has_noise + b.key.has_mask : 0;
    if (cudaMemcpyAsync(c->rows_dev, c->rows_host, n * P * 8, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(c->ptr_dev, c->ptr_host, (size_t)c->cap * PTR_PLANES * sizeof(void*),
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
        return LENSGB_ERR_CUDA;
    // PSFs gathered through the table: device-resident ones in place, host ones
    // from their pinned staging slots
    if (b.k2 > 0)
        table_copy((unsigned char*)c->psf_dev, c->ptr_dev + (size_t)PSF_PLANE * c->cap,
                   (size_t)b.k2 * b.esz, n, 0, st);
    int rc;
    if (!b.key.likelihood) {
        rc = lensgb_image(c->model, c->rows_dev, n, c->psf_dev, b.k2, c->img_dev, 0, st);
    } else {
        const size_t bytes = (size_t)b.npix * 8;
        int plane = 1;
        table_copy((unsigned char*)c->data_dev, c->ptr_dev + plane++ * c->cap, bytes, n, 0, st);
        if (c->noise_dev)
            table_copy((unsigned char*)c->noise_dev, c->ptr_dev + plane++ * c->cap, bytes, n, 0, st);
        if (c->mask_dev)
            table_copy((unsigned char*)c->mask_dev, c->ptr_dev + plane++ * c->cap, bytes, n, 0, st);
        lensgb_noise_desc nd;
        memset(&nd, 0, sizeof nd);
        nd.data_dev = c->data_dev;
        nd.data_stride = b.npix;
        nd.noise_map_dev = c->noise_dev;
        nd.noise_stride = c->noise_dev ? b.npix : 0;
        nd.mask_dev = c->mask_dev;
        nd.mask_stride = c->mask_dev ? b.npix : 0;
        nd.exposure_time = b.key.exposure_time;
        nd.background_rms = b.key.background_rms;
        rc = lensgb_loglike(c->model, c->rows_dev, n, c->psf_dev, b.k2, &nd, c->img_dev,
                            c->logl_dev, st);
        if (rc == LENSGB_OK && cudaMemcpyAsync(c->logl_host, c->logl_dev, n * 8,
                                               cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = LENSGB_ERR_CUDA;
    }
    if (rc) return rc;
    // every image to its request's host buffer (or the pinned staging)
    table_copy((unsigned char*)c->img_dev, c->ptr_dev, (size_t)b.npix * b.esz, n, 1, st);
    return cudaGetLastError() == cudaSuccess ? LENSGB_OK : LENSGB_ERR_CUDA;
}

// Runs the batch's launch sequence: eagerly the first time a context meets a
// launch shape `key`, then (use_graphs) captured into a CUDA graph and replayed.
int launch_or_replay(lensgb_server* s, Context* c, int n, long long key) {
    cudaStream_t st = c->stream;
    auto g = c->graphs.find(key);
    if (g != c->graphs.end()) {
        if (cudaGraphLaunch(g->second, st) != cudaSuccess) return LENSGB_ERR_CUDA;
        s->stats.graph_launches++;
        return LENSGB_OK;
    }
    if (!(s->cfg.use_graphs && c->eager_runs[key] >= 1)) {
        const int rc = launch_batch(s, c, n);
        if (rc == LENSGB_OK) c->eager_runs[key]++;
        return rc;
    }
    // the same context and shape ran eagerly before: capture and replay
    const long long tc = s->now();
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return LENSGB_ERR_CUDA;
    int rc = launch_batch(s, c, n);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc == LENSGB_OK && e == cudaSuccess && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
        c->graphs[key] = exec;
        s->stats.graph_captures++;
    } else {
        exec = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    s->stats.capture_ns += s->now() - tc;
    if (exec) {
        if (cudaGraphLaunch(exec, st) != cudaSuccess) return LENSGB_ERR_CUDA;
        s->stats.graph_launches++;
        return LENSGB_OK;
    }
    return launch_batch(s, c, n);  // capture failed: run eagerly
}

int run_batch(lensgb_server* s, Context* c, int n) {
    Bucket& b = *s->wb[c->bucket];
    cudaStream_t st = c->stream;
    // stage the small per-request inputs and the pointer tables in pinned memory
    const size_t P = (size_t)b.n_params;
    const size_t ib = (size_t)b.npix * b.esz;
    const size_t pb = (size_t)b.npix * 8;
    const int planes = b.key.likelihood ? 1 + b.key.has_noise + b.key.has_mask : 0;
    if (b.mixed) {
        c->grids.resize((size_t)n);
        long long po = 0, ko = 0;
        for (int i = 0; i < n; ++i) {
            const Req* q = c->batch[i];
            const lensgb_request& r = q->r;
            memcpy(c->rows_host + i * P, r.params, P * 8);
            if (q->k2 > 0) memcpy(c->psf_host + ko * b.esz, r.psf, (size_t)q->k2 * b.esz);
            lensgb_system_grid& gi = c->grids[(size_t)i];
            gi.nx = r.desc.nx;
            gi.ny = r.desc.ny;
            memcpy(gi.transform_pix2angle, r.desc.transform_pix2angle, sizeof gi.transform_pix2angle);
            gi.ra_at_xy_0 = r.desc.ra_at_xy_0;
            gi.dec_at_xy_0 = r.desc.dec_at_xy_0;
            gi.kernel_size = r.desc.kernel_size;
            gi.supersampling = r.desc.supersampling;
            c->boff_host[i] = po * (long long)b.esz;
            c->ptr_host[i] = (r.image_out && q->out_pinned) ? r.image_out
                                                             : (void*)(c->img_host + po * b.esz);
            po += q->npix;
            ko += q->k2;
        }
        c->boff_host[n] = po * (long long)b.esz;
        lensgb::MixedCounts mc;
        const bool conv = b.key.desc.psf_type != LENSGB_PSF_NONE;
        int rc = lensgb::mixed_fill(c->model, c->stage_host + c->o_tab, c->ml, c->grids.data(), n,
                                    conv, &mc);
        if (rc) return rc;
        // launch shape: CTA counts in power-of-two classes of the batch's tiles,
        // the supersampling and convolution groups present, and (run-time-width
        // group) the kernel width rounded up; one graph per shape
        auto p2 = [](int v, int cap) {
            int k = 0;
            while ((1 << k) < v && (1 << k) < cap) ++k;
            return k;
        };
        const int nsm = s->n_sms;
        lensgb::MixedGrid& gr = c->mgrid;
        int rtot = 0, rmask = 0;
        for (int g = 0; g < lensgb::MIX_RAY_GROUPS; ++g) rtot += mc.ray_tiles[g];
        const int kr = p2(rtot, 8 * nsm);
        for (int g = 0; g < lensgb::MIX_RAY_GROUPS; ++g) {
            gr.ray_ctas[g] = mc.ray_tiles[g] > 0 ? std::min(1 << kr, 8 * nsm) : 0;
            if (mc.ray_tiles[g] > 0) rmask |= 1 << g;
        }
        int ctot = 0, mask = 0, kvar = 0;
        for (int g = 0; g < 8; ++g) ctot += mc.conv_tiles[g];
        const int kc = p2(ctot, 4 * nsm);
        for (int g = 0; g < 8; ++g) {
            gr.conv_ctas[g] = 0;
            gr.conv_kmax[g] = 0;
            if (mc.conv_tiles[g] == 0) continue;
            mask |= 1 << g;
            gr.conv_ctas[g] = std::min(1 << kc, 4 * nsm);
            if (g >= 1 && g <= 6) {
                gr.conv_kmax[g] = 8 * g - 1;  // the widest odd kernel of the group
            } else {
                kvar = ((mc.kmax[g] + 15) / 16) * 16 - 1;
                gr.conv_kmax[g] = kvar;
            }
        }
        const long long key = (long long)mask | ((long long)kvar << 8) | ((long long)kr << 16) |
                              ((long long)kc << 24) | ((long long)rmask << 32);
        rc = launch_or_replay(s, c, n, key);
        if (rc) return rc;
        s->stats.mixed_batches++;
        return cudaEventRecord(c->done, st) == cudaSuccess ? LENSGB_OK : LENSGB_ERR_CUDA;
    }
    for (int i = 0; i < n; ++i) {
        const Req* q = c->batch[i];
        const lensgb_request& r = q->r;
        memcpy(c->rows_host + i * P, r.params, P * 8);
        if (b.k2 > 0) {
            void* kp = (void*)r.psf;
            if (!(q->in_pinned & 16)) {
                kp = c->psf_host + i * (size_t)b.k2 * b.esz;
                memcpy(kp, r.psf, (size_t)b.k2 * b.esz);
            }
            c->ptr_host[(size_t)PSF_PLANE * c->cap + i] = kp;
        }
        c->ptr_host[i] = (r.image_out && q->out_pinned) ? r.image_out : (void*)(c->img_host + i * ib);
        const void* src[3] = {r.data, r.noise_map, r.mask};
        const bool use[3] = {true, b.key.has_noise != 0, b.key.has_mask != 0};
        for (int k = 0, plane = 1; k < 3 && plane <= planes; ++k) {
            if (!use[k]) continue;
            void* p = (void*)src[k];
            if (!(q->in_pinned & (1 << k))) {
                // pageable input: stage it in pinned memory for the device to read
                p = c->in_host + ((size_t)(plane - 1) * c->cap + i) * pb;
                memcpy(p, src[k], pb);
            }
            c->ptr_host[(size_t)plane * c->cap + i] = p;
            ++plane;
        }
    }
    int rc = launch_or_replay(s, c, n, n);
    if (rc) return rc;
    if (cudaEventRecord(c->done, st) != cudaSuccess) return LENSGB_ERR_CUDA;
    return LENSGB_OK;
}

void finish_batch(lensgb_server* s, Context* c, int rc) {
    const long long t = s->now();
    Bucket& b = *s->wb[c->bucket];
    const size_t ib = (size_t)b.npix * b.esz;
    for (size_t i = 0; i < c->batch.size(); ++i) {
        Req* q = c->batch[i];
        if (rc == LENSGB_OK && b.key.likelihood && q->r.logl_out) *q->r.logl_out = c->logl_host[i];
        if (rc == LENSGB_OK && q->r.image_out && !q->out_pinned) {
            const size_t o = b.mixed ? (size_t)c->boff_host[i] : i * ib;
            memcpy(q->r.image_out, c->img_host + o, (size_t)q->npix * b.esz);
        }
        q->rc = rc;
        q->t_done = t;
        q->state.store(rc == LENSGB_OK ? LENSGB_REQ_DONE : LENSGB_REQ_FAILED,
                       std::memory_order_release);
    }
    s->n_done += (long long)c->batch.size();
    c->batch.clear();
    c->busy = false;
    c->last_used = t;
    s->inflight--;
}

// Ends the first m queued requests of a bucket with status rc (FAILED), except
// those a caller cancelled meanwhile (already ended and counted).
void fail_head(lensgb_server* s, Bucket& b, int m, int rc) {
    for (int i = 0; i < m && !b.queue.empty(); ++i) {
        Req* q = b.queue.front();
        b.queue.pop_front();
        int expected = LENSGB_REQ_QUEUED;
        if (!q->state.compare_exchange_strong(expected, LENSGB_REQ_RUNNING,
                                              std::memory_order_acq_rel))
            continue;
        q->rc = rc;
        q->t_done = s->now();
        q->state.store(LENSGB_REQ_FAILED, std::memory_order_release);
        s->n_done++;
    }
}

// Drops cancelled requests from the front of every bucket queue.
void drop_cancelled(lensgb_server* s) {
    for (Bucket* b : s->wb)
        while (!b->queue.empty() &&
               b->queue.front()->state.load(std::memory_order_acquire) == LENSGB_REQ_CANCELLED)
            b->queue.pop_front();
}

// Pick the bucket whose oldest waiting request is oldest and that can get a
// context; form and launch one batch.  Returns false if nothing was launched.
bool launch_one(lensgb_server* s) {
    drop_cancelled(s);
    int best = -1;
    long long best_t = 0;
    for (size_t k = 0; k < s->wb.size(); ++k) {
        Bucket& b = *s->wb[k];
        if (b.queue.empty()) continue;
        bool idle = false;
        for (Context* c : b.ctx) idle |= !c->busy;
        if (!idle && (int)b.ctx.size() >= s->cfg.contexts_per_bucket) continue;
        const long long t = b.queue.front()->t_release;
        if (best < 0 || t < best_t) {
            best = (int)k;
            best_t = t;
        }
    }
    if (best < 0) return false;
    Bucket& b = *s->wb[best];
    Context* c = nullptr;
    for (Context* x : b.ctx)
        if (!x->busy) {
            c = x;
            break;
        }
    const int n = (int)std::min<size_t>(b.queue.size(), (size_t)s->cfg.max_batch);
    // what the first m queued requests need (prefix sums over the queue head)
    auto& pp = s->pre_pix;
    auto& pk = s->pre_kel;
    pp.assign((size_t)n + 1, 0);
    pk.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i) {
        pp[(size_t)i + 1] = pp[(size_t)i] + b.queue[(size_t)i]->npix;
        pk[(size_t)i + 1] = pk[(size_t)i] + b.queue[(size_t)i]->k2;
    }
    auto need = [&](int m) { return Need{m, pp[(size_t)m], pk[(size_t)m]}; };
    if (!c) {
        if (!make_room(s, context_bytes(b, need(n)), nullptr) &&
            !make_room(s, context_bytes(b, need(1)), nullptr)) {
            if (s->inflight > 0) return false;  // wait for memory
            // nothing in flight can free memory and no idle context is left to
            // evict: the head request can never fit the budget (in a uniform
            // bucket, neither can any other of its queue)
            fail_head(s, b, b.mixed ? 1 : (int)b.queue.size(), LENSGB_ERR_OOM);
            return true;
        }
        c = new_context(s, best);
        if (!c) {
            // cannot build the model: fail the queued requests of this bucket
            fail_head(s, b, (int)b.queue.size(), LENSGB_ERR_UNSUPPORTED);
            return true;
        }
    }
    // the largest batch that fits the budget (halving from the queue length)
    int rc = LENSGB_ERR_OOM;
    for (int m = n; m >= 1 && rc == LENSGB_ERR_OOM; m = (m == 1 ? 0 : (m + 1) / 2))
        rc = grow_context(s, c, need(m));
    if (rc == LENSGB_ERR_OOM) {
        if (c->cap == 0 && s->inflight == 0) {
            // nothing in flight can free memory: the request can never fit (in a
            // uniform bucket, neither can any other of its queue)
            fail_head(s, b, b.mixed ? 1 : (int)b.queue.size(), LENSGB_ERR_OOM);
            return true;
        }
        return false;
    }
    // the longest queue head that the context holds
    int nb = std::min(n, c->cap);
    while (nb > 1 && (pp[(size_t)nb] > c->pix_cap || pk[(size_t)nb] > c->kel_cap)) --nb;
    const long long t = s->now();
    for (int i = 0; i < nb; ++i) {
        Req* q = b.queue.front();
        b.queue.pop_front();
        // admission and lensgb_server_cancel race for the QUEUED state
        int expected = LENSGB_REQ_QUEUED;
        if (!q->state.compare_exchange_strong(expected, LENSGB_REQ_RUNNING,
                                              std::memory_order_acq_rel))
            continue;  // cancelled
        q->t_admit = t;
        c->batch.push_back(q);
    }
    nb = (int)c->batch.size();
    if (nb == 0) return true;  // every request of the head was cancelled
    c->busy = true;
    c->last_used = t;
    s->inflight++;
    s->stats.batches++;
    s->stats.requests_launched += nb;
    const long long tl = s->now();
    rc = run_batch(s, c, nb);
    s->stats.host_launch_ns += s->now() - tl;
    if (rc != LENSGB_OK) {
        cudaStreamSynchronize(c->stream);
        cudaGetLastError();
        finish_batch(s, c, rc);
    }
    return true;
}

void worker_main(lensgb_server* s) {
    cudaSetDevice(s->device);
    std::vector<Req*> ready;
    while (!s->stop.load()) {
        bool progress = false;
        const long long t = s->now();
        {
            std::lock_guard<std::mutex> lock(s->mu);
            // release due requests in submission order
            auto& in = s->incoming;
            size_t w = 0;
            for (size_t i = 0; i < in.size(); ++i) {
                if (in[i]->t_release <= t)
                    ready.push_back(in[i]);
                else
                    in[w++] = in[i];
            }
            in.resize(w);
            while (s->wb.size() < s->buckets.size()) s->wb.push_back(s->buckets[s->wb.size()]);
        }
        for (Req* q : ready) s->wb[q->bucket]->queue.push_back(q);
        progress |= !ready.empty();
        ready.clear();
        // completions
        for (Context* c : s->contexts) {
            if (!c->busy) continue;
            cudaError_t e = cudaEventQuery(c->done);
            if (e == cudaSuccess) {
                finish_batch(s, c, LENSGB_OK);
                progress = true;
            } else if (e != cudaErrorNotReady) {
                cudaGetLastError();
                finish_batch(s, c, LENSGB_ERR_CUDA);
                progress = true;
            }
        }
        // admissions
        while (s->inflight < s->cfg.n_streams && launch_one(s)) progress = true;
        if (!progress) {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait_for(lock, std::chrono::microseconds(20));
        }
    }
    // drain what is in flight before the worker exits
    for (Context* c : s->contexts)
        if (c->busy) {
            cudaEventSynchronize(c->done);
            finish_batch(s, c, LENSGB_OK);
        }
}

// Memory the server's device reads and writes through the same address:
// page-locked (cudaHostAlloc / registered) host memory, managed memory, or
// device memory of that device (inputs kept resident on the GPU by the caller).
bool device_readable(const void* p, int device) {
    cudaPointerAttributes pa;
    bool ok = false;
    if (cudaPointerGetAttributes(&pa, p) == cudaSuccess) {
        ok = (pa.type == cudaMemoryTypeHost && pa.devicePointer == p) ||
             pa.type == cudaMemoryTypeManaged ||
             (pa.type == cudaMemoryTypeDevice && pa.device == device);
    }
    cudaGetLastError();
    return ok;
}

bool on_device(const void* p) {
    cudaPointerAttributes pa;
    const bool ok = cudaPointerGetAttributes(&pa, p) == cudaSuccess &&
                    pa.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    return ok;
}

// Requests that a mixed bucket can take: image only, no supersampled
// convolution, PSF in host memory.
bool mixable(const lensgb_server* s, const lensgb_request& r, bool psf_dev) {
    return s->cfg.mixed_grids && !r.data && !psf_dev &&
           !(r.desc.supersampling_convolution && r.desc.supersampling > 1);
}

int bucket_for(lensgb_server* s, const lensgb_request& r, bool psf_dev, int* out) {
    BucketKey k;
    memset(&k, 0, sizeof k);
    k.desc = r.desc;
    k.psf_on_device = psf_dev ? 1 : 0;
    k.likelihood = r.data ? 1 : 0;
    k.has_noise = r.data && r.noise_map ? 1 : 0;
    k.has_mask = r.data && r.mask ? 1 : 0;
    k.background_rms = r.data ? r.background_rms : 0.0;
    k.exposure_time = r.data ? r.exposure_time : 0.0;
    auto it = s->bucket_index.find(k);
    if (it != s->bucket_index.end()) {
        *out = it->second;
        return LENSGB_OK;
    }
    // validate the model once per exact key
    lensgb_model* m = nullptr;
    int rc = lensgb_model_create(&r.desc, &m);
    if (rc) return serr(rc, std::string("request model: ") + lensgb_last_error());
    const int n_params = lensgb_model_param_count(m);
    lensgb_model_destroy(m);
    const bool mixed = mixable(s, r, psf_dev);
    BucketKey bk = k;
    if (mixed) {
        // the bucket's model: the request's profile stack, precision, PSF type
        // (and, with mixed_grids == 1, supersampling) on a 1 x 1 placeholder
        // grid; lensgb_image_mixed takes every system's grid, supersampling and
        // PSF size from its table
        lensgb_model_desc& d = bk.desc;
        d.nx = d.ny = 1;
        if (s->cfg.mixed_grids >= 2) d.supersampling = 1;
        d.transform_pix2angle[0] = d.transform_pix2angle[3] = 1.0;
        d.transform_pix2angle[1] = d.transform_pix2angle[2] = 0.0;
        d.ra_at_xy_0 = d.dec_at_xy_0 = 0.0;
        d.kernel_size = d.psf_type == LENSGB_PSF_NONE ? 0 : 1;
        d.supersampling_convolution = 0;
        d.low_res_kernel_size = 0;
        auto mi = s->mixed_index.find(bk);
        if (mi != s->mixed_index.end()) {
            *out = mi->second;
            s->bucket_index[k] = *out;
            return LENSGB_OK;
        }
    }
    Bucket* b = new Bucket();
    b->key = bk;
    b->mixed = mixed;
    b->n_params = n_params;
    b->npix = (long long)r.desc.nx * r.desc.ny;
    b->k2 = r.desc.psf_type == LENSGB_PSF_NONE
                ? 0
                : r.desc.kernel_size * r.desc.kernel_size +
                      r.desc.low_res_kernel_size * r.desc.low_res_kernel_size;
    b->esz = r.desc.precision == LENSGB_FP64 ? 8 : 4;
    s->buckets.push_back(b);
    *out = (int)s->buckets.size() - 1;
    s->bucket_index[k] = *out;
    if (mixed) s->mixed_index[bk] = *out;
    return LENSGB_OK;
}

}  // namespace

extern "C" {

int lensgb_server_create(const lensgb_server_config* cfg, lensgb_server** out) {
    if (!out) return serr(LENSGB_ERR_INVALID, "null output handle pointer");
    *out = nullptr;
    lensgb_server_config c;
    memset(&c, 0, sizeof c);
    if (cfg) c = *cfg;
    if (c.n_streams <= 0) c.n_streams = 4;
    if (c.max_batch <= 0) c.max_batch = 256;
    if (c.contexts_per_bucket <= 0) c.contexts_per_bucket = 2;
    if (c.hbm_budget_bytes <= 0) c.hbm_budget_bytes = 4ll << 30;
    if (c.n_streams > 64 || c.max_batch > 65535 || c.contexts_per_bucket > 16)
        return serr(LENSGB_ERR_INVALID, "n_streams <= 64, max_batch <= 65535, "
                                        "contexts_per_bucket <= 16");
    if (c.mixed_grids < 0 || c.mixed_grids > 2)
        return serr(LENSGB_ERR_INVALID, "mixed_grids must be 0, 1 or 2");
    lensgb_server* s = new lensgb_server();
    s->cfg = c;
    cudaGetDevice(&s->device);
    s->n_sms = lensgb::num_sms();
    memset(&s->stats, 0, sizeof s->stats);
    s->t0 = Clock::now();
    s->worker = std::thread(worker_main, s);
    *out = s;
    return LENSGB_OK;
}

long long lensgb_server_clock_ns(const lensgb_server* s) { return s ? s->now() : -1; }

int lensgb_server_submit(lensgb_server* s, const lensgb_request* reqs, int n, long long* tickets) {
    if (!s) return serr(LENSGB_ERR_INVALID, "null server");
    if (n < 0 || (n > 0 && (!reqs || !tickets)))
        return serr(LENSGB_ERR_INVALID, "null request array or tickets");
    // validation and pointer queries outside the lock the worker needs
    std::vector<int> pinned((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        const lensgb_request& r = reqs[i];
        if (!r.params) return serr(LENSGB_ERR_INVALID, "request without params");
        if (r.desc.psf_type != LENSGB_PSF_NONE && !r.psf)
            return serr(LENSGB_ERR_INVALID, "request without a PSF kernel");
        if (r.data && r.noise_map == nullptr && !(r.exposure_time > 0))
            return serr(LENSGB_ERR_INVALID, "likelihood request needs exposure_time > 0");
        const void* in[3] = {r.data, r.noise_map, r.mask};
        for (int k = 0; k < 3; ++k)
            if (in[k] && device_readable(in[k], s->device)) pinned[(size_t)i] |= 1 << k;
        if (r.image_out && device_readable(r.image_out, s->device)) pinned[(size_t)i] |= 8;
        if (r.psf && on_device(r.psf)) {
            if (!device_readable(r.psf, s->device))
                return serr(LENSGB_ERR_INVALID, "PSF kernel in another device's memory");
            pinned[(size_t)i] |= 16 | 32;  // 32: the PSF is in device memory
        }
    }
    // enqueue in chunks, so that a large submission does not stall the worker
    constexpr int CHUNK = 256;
    for (int i0 = 0; i0 < n; i0 += CHUNK) {
        std::lock_guard<std::mutex> lock(s->mu);
        const long long t = s->now();
        for (int i = i0; i < n && i < i0 + CHUNK; ++i) {
            const lensgb_request& r = reqs[i];
            int bucket = -1;
            int rc = bucket_for(s, r, (pinned[(size_t)i] & 32) != 0, &bucket);
            if (rc) return rc;
            s->reqs.emplace_back();
            Req& q = s->reqs.back();
            q.r = r;
            q.ticket = (long long)s->reqs.size() - 1;
            q.bucket = bucket;
            q.t_submit = t;
            q.t_release = r.release_ns > t ? r.release_ns : t;
            q.out_pinned = (pinned[(size_t)i] & 8) != 0;
            q.in_pinned = pinned[(size_t)i] & 23;
            q.npix = (long long)r.desc.nx * r.desc.ny;
            q.k2 = r.desc.psf_type == LENSGB_PSF_NONE
                       ? 0
                       : r.desc.kernel_size * r.desc.kernel_size +
                             r.desc.low_res_kernel_size * r.desc.low_res_kernel_size;
            s->incoming.push_back(&q);
            tickets[i] = q.ticket;
        }
        s->cv.notify_one();
    }
    return LENSGB_OK;
}

int lensgb_server_poll(lensgb_server* s, long long ticket, int* state) {
    if (!s || !state) return serr(LENSGB_ERR_INVALID, "null server or state");
    Req* q;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (ticket < 0 || ticket >= (long long)s->reqs.size())
            return serr(LENSGB_ERR_INVALID, "unknown ticket");
        q = &s->reqs[(size_t)ticket];
    }
    *state = q->state.load(std::memory_order_acquire);
    return *state == LENSGB_REQ_FAILED ? q->rc : LENSGB_OK;
}

int lensgb_server_cancel(lensgb_server* s, long long ticket, int* cancelled) {
    if (!s) return serr(LENSGB_ERR_INVALID, "null server");
    Req* q;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (ticket < 0 || ticket >= (long long)s->reqs.size())
            return serr(LENSGB_ERR_INVALID, "unknown ticket");
        q = &s->reqs[(size_t)ticket];
    }
    int expected = LENSGB_REQ_QUEUED;
    const bool ok = q->state.compare_exchange_strong(expected, LENSGB_REQ_CANCELLED,
                                                     std::memory_order_acq_rel);
    if (ok) {
        q->t_done = s->now();
        s->n_done++;
        s->cv.notify_one();
    }
    if (cancelled) *cancelled = ok ? 1 : 0;
    return LENSGB_OK;
}

int lensgb_server_wait(lensgb_server* s, long long ticket, double timeout_s, int* state) {
    if (!s || !state) return serr(LENSGB_ERR_INVALID, "null server or state");
    const auto until = Clock::now() + std::chrono::duration<double>(timeout_s);
    for (;;) {
        int rc = lensgb_server_poll(s, ticket, state);
        if (rc || *state == LENSGB_REQ_DONE || *state == LENSGB_REQ_CANCELLED) return rc;
        if (Clock::now() > until) return LENSGB_OK;
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

int lensgb_server_drain(lensgb_server* s, double timeout_s) {
    if (!s) return serr(LENSGB_ERR_INVALID, "null server");
    const auto until = Clock::now() + std::chrono::duration<double>(timeout_s);
    for (;;) {
        long long total;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            total = (long long)s->reqs.size();
        }
        if (s->n_done.load() >= total) return LENSGB_OK;
        if (Clock::now() > until) return serr(LENSGB_ERR_CUDA, "drain timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int lensgb_server_request_times(lensgb_server* s, long long ticket, long long* release_ns,
                                long long* admit_ns, long long* done_ns) {
    if (!s) return serr(LENSGB_ERR_INVALID, "null server");
    Req* q;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (ticket < 0 || ticket >= (long long)s->reqs.size())
            return serr(LENSGB_ERR_INVALID, "unknown ticket");
        q = &s->reqs[(size_t)ticket];
    }
    const int st = q->state.load(std::memory_order_acquire);
    if (release_ns) *release_ns = q->t_release;
    if (admit_ns)
        *admit_ns = st >= LENSGB_REQ_RUNNING && st != LENSGB_REQ_CANCELLED ? q->t_admit : -1;
    if (done_ns) *done_ns = st >= LENSGB_REQ_DONE ? q->t_done : -1;
    return LENSGB_OK;
}

int lensgb_server_get_stats(lensgb_server* s, lensgb_server_stats* out) {
    if (!s || !out) return serr(LENSGB_ERR_INVALID, "null server or stats");
    // read on the caller's thread while the worker runs: the counters are
    // monotone and only approximately consistent with each other
    *out = s->stats;
    out->bytes_held = (long long)s->bytes_held;
    out->peak_bytes = (long long)s->peak_bytes;
    out->requests_done = s->n_done.load();
    return LENSGB_OK;
}

int lensgb_server_destroy(lensgb_server* s) {
    if (!s) return LENSGB_OK;
    s->stop.store(true);
    s->cv.notify_one();
    if (s->worker.joinable()) s->worker.join();
    for (Context* c : s->contexts) destroy_context(s, c);
    for (Bucket* b : s->buckets) delete b;
    delete s;
    return LENSGB_OK;
}

}  // extern "C"
