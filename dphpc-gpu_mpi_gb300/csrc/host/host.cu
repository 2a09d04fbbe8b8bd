// host.cu — host side of libgpumpi.so: the C ABI of include/gpumpi.h.
//
// Replaces the reference's host launcher and harness (gpu_libs/gpu_main/main.cu:133-320,
// tests/test_runner.cuh:26-86): option parsing, device-memory layout of all runtime state (no managed
// memory), per-launch reset, cooperative launch of the persistent rank kernel with occupancy-derived
// geometry, collection of device-side error records, and staging of host buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../programs/rt_kernel.cuh"
#include "../runtime/rt_core.cuh"
#include "host_io.h"

using gpumpi::Runtime;

extern const gpumpi_prog_entry g_test_programs[];
extern const int g_num_test_programs;
extern const gpumpi_prog_entry g_hot_programs[];
extern const int g_num_hot_programs;
extern const gpumpi_prog_entry g_app_programs[];
extern const int g_num_app_programs;
// a converted program's table (csrc/host/user_main.cu), present only in executables built around one
extern const gpumpi_prog_entry g_user_programs[] __attribute__((weak));
extern const int g_num_user_programs __attribute__((weak));

extern "C" cudaError_t gpumpi_internal_install(Runtime* d_rt, MPI_Comm world, MPI_Group gworld, MPI_Group gempty,
                                                cudaStream_t stream);
extern "C" cudaError_t gpumpi_internal_install_dev(const Runtime* d_rt, const void* const* d_vals, cudaStream_t stream);

namespace {

std::atomic<long long> g_launches{0};
std::string g_create_error;
std::mutex g_limits_mu;
bool g_limits_set = false;

const gpumpi_prog_entry* find_program(int id) {
    for (int i = 0; i < g_num_test_programs; i++)
        if (g_test_programs[i].id == id) return &g_test_programs[i];
    for (int i = 0; i < g_num_hot_programs; i++)
        if (g_hot_programs[i].id == id) return &g_hot_programs[i];
    for (int i = 0; i < g_num_app_programs; i++)
        if (g_app_programs[i].id == id) return &g_app_programs[i];
    if (&g_num_user_programs != nullptr && g_user_programs != nullptr)
        for (int i = 0; i < g_num_user_programs; i++)
            if (g_user_programs[i].id == id) return &g_user_programs[i];
    return nullptr;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// carve sub-allocations out of one region
struct Carver {
    size_t off = 0;
    template <class T>
    size_t take(size_t count, size_t align = 256) {
        off = align_up(off, align);
        size_t o = off;
        off += sizeof(T) * count;
        return o;
    }
};

// small state re-uploaded before every launch (everything else in the control region is zeroed)
struct FixedImage {
    MPI_Comm_impl world;
    gpumpi::Board board;
    MPI_Group_impl gworld;
    MPI_Group_impl gempty;
    unsigned ctx_counter;
};

}  // namespace

struct gpumpi_world {
    gpumpi_config cfg;
    int device = 0, sm_count = 0, max_blocks = 0;
    int T = 0, nengines = 0, blocks_per_sm = 0;
    size_t dyn_smem = 0;
    Runtime h_rt;
    Runtime* d_rt = nullptr;
    char* d_ctrl = nullptr;
    size_t ctrl_bytes = 0;
    char* d_data = nullptr;
    size_t data_bytes = 0;
    FixedImage* d_fixed = nullptr;
    FixedImage h_fixed;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0;
    int variant_override = -1, selector_mode = 3;
    int tune_vec = 0, tune_group = 0;
    // dynamic shared memory per block at most (-1: no cap).  What a block does not take as shared memory
    // stays L1 cache, which holds the executors' spilled registers and the ranks' private state:
    // measured at 1024 ranks, an 8 KiB cap instead of the ~18 KiB left over raises Allreduce from
    // 4.9 to 5.6 TB/s and uneven Alltoallv from 3.0 to 4.0 TB/s.
    long long dyn_smem_cap = 8192;
    // pinned host buffers: 1 = the kernel reads and writes them in place (device alias of the page-locked
    // allocation, every byte crosses the host link once); 0 = staged through device memory by copies
    // before and after the kernel; 2..4: an Allreduce between host buffers is cut into column slices so
    // both directions of the host link carry data at once (allreduce_host_sliced), other calls treat 2..4
    // as 1.  Measured at 1024 ranks x 1 MiB fp32 Allreduce with page-locked buffers (GB/s of 2 x payload,
    // host link: 211 GB/s host to device, 194 back, 343 both at once): in place 208, staged 193, slices of
    // 256 KiB per rank 266 (mode 2) / 266 (mode 3) / 258 (mode 4); 128 KiB slices 207-224, 64 KiB 174-186
    // (2D copies of narrow rows lose most of the two-way overlap).
    int host_direct = 3;
    bool host_aliased = false;  // the launch being prepared reads host memory in place: no bulk copies
    long long host_slice_bytes = 0;  // column slice per rank of the sliced path, bytes (0 = auto)
    int host_streams = 1;            // copy streams per direction of the sliced path (row groups)
    cudaStream_t xs_in[4] = {}, xs_out[4] = {};  // the sliced path's copy streams (created on first use)
    cudaEvent_t xev[4] = {};                         // input copied, slice folded, call start, call end
    signed char* d_table = nullptr;
    float* d_mlp = nullptr;
    // scratch for host-buffer staging
    void* d_stage[8] = {};
    size_t stage_bytes[8] = {};
    // host mirrors of the error/exit records
    std::vector<gpumpi::ErrorRecord> h_err;
    std::vector<int> h_exit;
    HostService* hio = nullptr;  // the device -> host channel's service thread and mapped memory
};

#define CK(expr)                                                                               \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            if (w) w->err = std::string(#expr) + ": " + cudaGetErrorString(e_);                \
            return GPUMPI_ERR_CUDA;                                                            \
        }                                                                                      \
    } while (0)

extern "C" {

int gpumpi_config_init(gpumpi_config* c) {
    if (!c) return GPUMPI_ERR_ARG;
    memset(c, 0, sizeof(*c));
    c->nranks = 1;
    c->threads_per_block = 0;
    c->engine_blocks = -1;
    c->pending_requests = 1024;   // reference CLI default (main.cu:76)
    c->mailbox_depth = 64;
    c->unexpected_depth = 256;
    c->eager_bytes = 1024;
    c->max_types = 16;
    c->posted_depth = 1024;
    c->device = 0;
    c->stack_bytes = 8192;
    c->heap_bytes = 0;
    c->arena_bytes = 64ull << 20;
    c->copy_chunk_bytes = 256 << 10;
    c->engine_min_bytes = 256 << 10;
    c->timeout_s = 20.0;
    c->trace_capacity = 0;
    return GPUMPI_SUCCESS;
}

// ---gpumpi -n <ranks> -g <blocks> -b <threads> -s <stack> -p <heap> -e <pending>  (main.cu:70-78)
int gpumpi_parse_args(int argc, char** argv, gpumpi_config* cfg) {
    int pos = -1;
    for (int i = 0; i < argc; i++)
        if (strcmp(argv[i], "---gpumpi") == 0) pos = i;
    if (pos < 0) return -1;
    long long g = 0;
    for (int i = pos + 1; i + 1 < argc; i += 2) {
        const char* k = argv[i];
        long long v = atoll(argv[i + 1]);
        if (!strcmp(k, "-n") || !strcmp(k, "--numProcs")) cfg->nranks = (int)v;
        else if (!strcmp(k, "-g") || !strcmp(k, "--blocksPerGrid")) g = v;
        else if (!strcmp(k, "-b") || !strcmp(k, "--threadsPerBlock")) cfg->threads_per_block = (int)v;
        else if (!strcmp(k, "-s") || !strcmp(k, "--stackSize")) cfg->stack_bytes = (size_t)v;
        else if (!strcmp(k, "-p") || !strcmp(k, "--heapSize")) cfg->heap_bytes = (size_t)v;
        else if (!strcmp(k, "-e") || !strcmp(k, "--pendingBufferSize")) cfg->pending_requests = (int)v;
        else if (!strcmp(k, "--engines")) cfg->engine_blocks = (int)v;
        else if (!strcmp(k, "--timeout")) cfg->timeout_s = atof(argv[i + 1]);
    }
    // a rank is a block here, so -g alone (the reference's blocks-per-grid) also gives the rank count
    if (cfg->nranks <= 1 && g > 0) cfg->nranks = (int)g;
    return pos;
}

const char* gpumpi_last_error(gpumpi_world* w) { return w ? w->err.c_str() : g_create_error.c_str(); }

long long gpumpi_kernel_launches(void) { return g_launches.load(); }

int gpumpi_world_create(const gpumpi_config* cfg_in, gpumpi_world** out) {
    gpumpi_world* w = nullptr;
    if (!cfg_in || !out) return GPUMPI_ERR_ARG;
    gpumpi_config cfg = *cfg_in;
    if (cfg.nranks < 1) {
        g_create_error = "nranks must be >= 1";
        return GPUMPI_ERR_ARG;
    }
    if (cfg.threads_per_block > 0 && (cfg.threads_per_block % 32 != 0 || cfg.threads_per_block > 256)) {
        // block tasks scan and copy with whole warps; the kernel is compiled for at most 256 threads
        g_create_error = "threads_per_block must be a multiple of 32 in [32, 256]";
        return GPUMPI_ERR_ARG;
    }
    if (cfg.eager_bytes < 16) cfg.eager_bytes = 16;
    cfg.eager_bytes = (cfg.eager_bytes + 15) & ~15;
    int md = 1;
    while (md < cfg.mailbox_depth) md <<= 1;
    cfg.mailbox_depth = md;
    if (cfg.unexpected_depth < 1) cfg.unexpected_depth = 1;
    if (cfg.posted_depth < 1) cfg.posted_depth = 1;
    if (cfg.pending_requests < 1) cfg.pending_requests = 1;
    if (cfg.max_types < 1) cfg.max_types = 1;
    if (cfg.timeout_s <= 0) cfg.timeout_s = 20.0;

    cudaError_t e = cudaSetDevice(cfg.device);
    if (e != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return GPUMPI_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lk(g_limits_mu);
        if (!g_limits_set) {
            cudaDeviceSetLimit(cudaLimitStackSize, cfg.stack_bytes);
            cudaDeviceSetLimit(cudaLimitMallocHeapSize, cfg.heap_bytes ? cfg.heap_bytes : (1ull << 30));
            cudaGetLastError();
            g_limits_set = true;
        }
    }
    w = new gpumpi_world();
    w->cfg = cfg;
    w->device = cfg.device;
    CK(cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, cfg.device));
    w->max_blocks = w->sm_count * 32;
    const int n = cfg.nranks;
    const int nb = w->max_blocks > n ? w->max_blocks : n;

    // ---- control region: zeroed before every launch ----
    Carver cc;
    size_t o_ranks = cc.take<gpumpi::RankState>(n);
    size_t o_ring = cc.take<gpumpi::Envelope>((size_t)n * cfg.mailbox_depth);
    size_t o_types = cc.take<gpumpi::TypeDesc>((size_t)n * cfg.max_types);
    size_t o_errors = cc.take<gpumpi::ErrorRecord>(nb);
    size_t o_exit = cc.take<int>(n);
    size_t o_arena_top = cc.take<unsigned long long>(1);
    size_t o_done = cc.take<unsigned>(1);
    size_t o_abort = cc.take<unsigned>(1);
    size_t o_trace_count = cc.take<unsigned long long>(1);
    const int tree_flags_cap = 1 << 16;
    size_t o_tree_flags = cc.take<unsigned>(tree_flags_cap);
    w->ctrl_bytes = align_up(cc.off, 256);

    // ---- data region ----
    Carver dc;
    size_t o_ring_pl = dc.take<unsigned char>((size_t)n * cfg.mailbox_depth * cfg.eager_bytes);
    size_t o_uq = dc.take<gpumpi::UqEntry>((size_t)n * cfg.unexpected_depth);
    size_t o_uq_pl = dc.take<unsigned char>((size_t)n * cfg.unexpected_depth * cfg.eager_bytes);
    size_t o_uq_free = dc.take<int>((size_t)n * cfg.unexpected_depth);
    size_t o_reqs = dc.take<MPI_Request_impl>((size_t)n * cfg.pending_requests);
    size_t o_req_free = dc.take<int>((size_t)n * cfg.pending_requests);
    size_t o_posted = dc.take<int>((size_t)n * cfg.posted_depth);
    size_t o_tasks = dc.take<gpumpi::Task>(nb);
    size_t o_wmembers = dc.take<int>(n);
    size_t o_wslots = dc.take<gpumpi::CollSlot>(n);
    size_t o_wtiny = dc.take<unsigned char>(2 * (size_t)gpumpi::TINY_BYTES * n);
    size_t o_board_ring = dc.take<gpumpi::BoardEntry>(4096);
    size_t o_trace = dc.take<gpumpi::TraceRec>(cfg.trace_capacity > 0 ? cfg.trace_capacity : 1);
    size_t o_arena = dc.take<unsigned char>(cfg.arena_bytes);
    // each rank's scratch pool (groups, staged thread-local buffers): room for four groups of the whole world
    const size_t scratch_pool_bytes = align_up(std::max<size_t>(4096, 4 * (sizeof(int) * (size_t)n + 128)), 256);
    size_t o_pool = dc.take<unsigned char>(scratch_pool_bytes * (size_t)n);
    const size_t tree_bytes = 64ull << 20;
    size_t o_tree = dc.take<unsigned char>(tree_bytes);
    size_t o_selc = dc.take<gpumpi::SelCacheRec>(n);
    size_t o_hio_tail = dc.take<unsigned long long>(1);
    size_t o_hio_broken = dc.take<unsigned>(n);
    w->data_bytes = align_up(dc.off, 256);

    CK(cudaMalloc(&w->d_ctrl, w->ctrl_bytes));
    CK(cudaMalloc(&w->d_data, w->data_bytes));
    CK(cudaMalloc(&w->d_fixed, sizeof(FixedImage)));
    CK(cudaMalloc(&w->d_rt, sizeof(Runtime)));
    CK(cudaMemset(w->d_data, 0, w->data_bytes));
    CK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&w->ev0));
    CK(cudaEventCreate(&w->ev1));

    // identity member list of the world
    std::vector<int> ident(n);
    for (int i = 0; i < n; i++) ident[i] = i;
    CK(cudaMemcpy(w->d_data + o_wmembers, ident.data(), sizeof(int) * n, cudaMemcpyHostToDevice));

    Runtime& r = w->h_rt;
    memset(&r, 0, sizeof(r));
    r.nranks = n;
    r.pending = cfg.pending_requests;
    r.mbox_depth = cfg.mailbox_depth;
    r.uq_depth = cfg.unexpected_depth;
    r.eager = cfg.eager_bytes;
    r.posted_cap = cfg.posted_depth;
    r.max_types = cfg.max_types;
    r.uq_payload_slots = cfg.unexpected_depth;
    r.timeout_ns = (long long)(cfg.timeout_s * 1e9);
    r.copy_chunk_bytes = cfg.copy_chunk_bytes;
    r.engine_min_bytes = cfg.engine_min_bytes;
    r.static_fold_bytes = 4096;
    r.static_bcast_bytes = 64 << 10;
    r.static_pull_bytes = 128 << 10;
    r.pull_chunks = 2;
    r.variant_override = -1;
    r.selector_mode = 0;
    r.trace_cap = cfg.trace_capacity;
    r.trace_enabled = cfg.trace_capacity > 0;
    r.ranks = (gpumpi::RankState*)(w->d_ctrl + o_ranks);
    r.sel_cache = (gpumpi::SelCacheRec*)(w->d_data + o_selc);
    // the device -> host channel: mapped ring, responses and windows, and the world's service thread
    if (cfg.host_window_bytes >= 0) {
        long long win = cfg.host_window_bytes;
        if (win == 0) win = std::min<long long>(1 << 20, std::max<long long>(4096, (16LL << 20) / n));
        win = std::max<long long>(4096, win & ~4095LL);
        w->hio = hio_create(n, (size_t)win, (unsigned long long*)(w->d_data + o_hio_tail),
                            (unsigned*)(w->d_data + o_hio_broken), &r.hio, &w->err);
        if (!w->hio) {
            g_create_error = w->err;
            gpumpi_world_destroy(w);
            return GPUMPI_ERR_NO_MEM;
        }
    }
    r.sel_epoch = 1;  // the data region starts zeroed: epoch 0 records are never valid
    r.ring = (gpumpi::Envelope*)(w->d_ctrl + o_ring);
    r.types = (gpumpi::TypeDesc*)(w->d_ctrl + o_types);
    r.errors = (gpumpi::ErrorRecord*)(w->d_ctrl + o_errors);
    r.exit_codes = (int*)(w->d_ctrl + o_exit);
    r.arena_top = (unsigned long long*)(w->d_ctrl + o_arena_top);
    r.ranks_done = (unsigned*)(w->d_ctrl + o_done);
    r.abort_flag = (unsigned*)(w->d_ctrl + o_abort);
    r.trace_count = (unsigned long long*)(w->d_ctrl + o_trace_count);
    r.scratch_pool = (unsigned char*)(w->d_data + o_pool);
    r.scratch_pool_bytes = (long long)scratch_pool_bytes;
    r.ring_payload = (unsigned char*)(w->d_data + o_ring_pl);
    r.uq = (gpumpi::UqEntry*)(w->d_data + o_uq);
    r.uq_payload = (unsigned char*)(w->d_data + o_uq_pl);
    r.uq_free = (int*)(w->d_data + o_uq_free);
    r.reqs = (MPI_Request_impl*)(w->d_data + o_reqs);
    r.req_free = (int*)(w->d_data + o_req_free);
    r.posted = (int*)(w->d_data + o_posted);
    r.tasks = (gpumpi::Task*)(w->d_data + o_tasks);
    r.world_members = (int*)(w->d_data + o_wmembers);
    r.world_slots = (gpumpi::CollSlot*)(w->d_data + o_wslots);
    r.trace = (gpumpi::TraceRec*)(w->d_data + o_trace);
    r.arena = (unsigned char*)(w->d_data + o_arena);
    r.arena_bytes = cfg.arena_bytes;
    r.tree_scratch = (unsigned char*)(w->d_data + o_tree);
    r.tree_scratch_bytes = (long long)tree_bytes;
    r.tree_flags = (unsigned*)(w->d_ctrl + o_tree_flags);
    r.tree_flags_cap = tree_flags_cap;
    r.world = &w->d_fixed->world;
    r.board = &w->d_fixed->board;
    r.ctx_counter = &w->d_fixed->ctx_counter;

    FixedImage& f = w->h_fixed;
    memset(&f, 0, sizeof(f));
    f.world.size = n;
    f.world.ctx = 1;  // the reference's MPI_COMM_WORLD context (communicator.cu:60)
    f.world.is_world = 1;
    f.world.magic = gpumpi::COMM_MAGIC;
    f.world.members = r.world_members;
    f.world.rank_of = nullptr;
    f.world.slots = r.world_slots;
    f.world.tiny = (unsigned char*)(w->d_data + o_wtiny);
    f.board.ring = (gpumpi::BoardEntry*)(w->d_data + o_board_ring);
    f.board.cap = 4096;
    f.gworld.size = n;
    f.gworld.ranks = r.world_members;
    f.gworld.refcount = 1;
    f.gworld.is_static = 1;
    f.gempty.size = 0;
    f.gempty.ranks = nullptr;
    f.gempty.refcount = 1;
    f.gempty.is_static = 1;
    f.ctx_counter = 2;
    w->h_err.resize(nb);
    w->h_exit.resize(n);
    *out = w;
    return GPUMPI_SUCCESS;
}

int gpumpi_world_destroy(gpumpi_world* w) {
    if (!w) return GPUMPI_SUCCESS;
    cudaSetDevice(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    hio_destroy(w->hio);
    cudaFree(w->d_ctrl);
    cudaFree(w->d_data);
    cudaFree(w->d_fixed);
    cudaFree(w->d_rt);
    cudaFree(w->d_table);
    cudaFree(w->d_mlp);
    for (auto& p : w->d_stage) cudaFree(p);
    for (auto* xs : {w->xs_in, w->xs_out})
        for (int k = 0; k < 4; k++)
            if (xs[k]) cudaStreamSynchronize(xs[k]), cudaStreamDestroy(xs[k]);
    for (auto& e : w->xev)
        if (e) cudaEventDestroy(e);
    if (w->ev0) cudaEventDestroy(w->ev0);
    if (w->ev1) cudaEventDestroy(w->ev1);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return GPUMPI_SUCCESS;
}

int gpumpi_world_get_info(gpumpi_world* w, gpumpi_world_info* info) {
    if (!w || !info) return GPUMPI_ERR_ARG;
    info->nranks = w->cfg.nranks;
    info->threads_per_block = w->T;
    info->engine_blocks = w->nengines;
    info->blocks_per_sm = w->blocks_per_sm;
    info->sm_count = w->sm_count;
    info->device = w->device;
    info->device_bytes = w->ctrl_bytes + w->data_bytes;
    return GPUMPI_SUCCESS;
}

int gpumpi_set_policy(gpumpi_world* w, int variant, int mode) {
    if (!w) return GPUMPI_ERR_ARG;
    w->h_rt.sel_epoch++;
    w->variant_override = variant;
    w->selector_mode = mode;
    return GPUMPI_SUCCESS;
}

int gpumpi_set_tuning(gpumpi_world* w, int key, long long value) {
    if (!w) return GPUMPI_ERR_ARG;
    w->h_rt.sel_epoch++;
    switch (key) {
    case GPUMPI_TUNE_VEC: w->tune_vec = (int)value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_DYN_SMEM: w->dyn_smem_cap = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_DIRECT:
        if (value < 0 || value > 4) return GPUMPI_ERR_ARG;
        w->host_direct = (int)value;
        return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_SLICE:
        if (value < 0) return GPUMPI_ERR_ARG;
        w->host_slice_bytes = value;
        return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_STREAMS:
        if (value < 1 || value > 4) return GPUMPI_ERR_ARG;
        w->host_streams = (int)value;
        return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STAGE_GROUP: w->tune_group = (int)value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_ENGINES: w->cfg.engine_blocks = (int)value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_COPY_CHUNK: w->h_rt.copy_chunk_bytes = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_ENGINE_MIN_BYTES: w->h_rt.engine_min_bytes = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_FOLD: w->h_rt.static_fold_bytes = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_BCAST: w->h_rt.static_bcast_bytes = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_PULL: w->h_rt.static_pull_bytes = value; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_PULL_CHUNKS:
        if (value < 1 || value > 64) return GPUMPI_ERR_ARG;
        w->h_rt.pull_chunks = (int)value;
        return GPUMPI_SUCCESS;
    // the learned policy's cached choices include the margin rule: a new margin starts a new epoch
    case GPUMPI_TUNE_MLP_MARGIN:
        w->h_rt.mlp_margin = (float)value * 1e-3f;
        w->h_rt.sel_epoch++;
        return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_MLP_MARGIN_PULL:
        w->h_rt.mlp_margin_pull = (float)value * 1e-3f;
        w->h_rt.sel_epoch++;
        return GPUMPI_SUCCESS;
    default: return GPUMPI_ERR_ARG;
    }
}

int gpumpi_get_tuning(gpumpi_world* w, int key, long long* value) {
    if (!w || !value) return GPUMPI_ERR_ARG;
    switch (key) {
    case GPUMPI_TUNE_VEC: *value = w->tune_vec; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_DYN_SMEM: *value = w->dyn_smem_cap; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_DIRECT: *value = w->host_direct; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_SLICE: *value = w->host_slice_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_HOST_STREAMS: *value = w->host_streams; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STAGE_GROUP: *value = w->tune_group; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_ENGINES: *value = w->cfg.engine_blocks; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_COPY_CHUNK: *value = w->h_rt.copy_chunk_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_ENGINE_MIN_BYTES: *value = w->h_rt.engine_min_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_FOLD: *value = w->h_rt.static_fold_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_BCAST: *value = w->h_rt.static_bcast_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_STATIC_PULL: *value = w->h_rt.static_pull_bytes; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_PULL_CHUNKS: *value = w->h_rt.pull_chunks; return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_MLP_MARGIN: *value = (long long)(w->h_rt.mlp_margin * 1e3f + 0.5f); return GPUMPI_SUCCESS;
    case GPUMPI_TUNE_MLP_MARGIN_PULL: *value = (long long)(w->h_rt.mlp_margin_pull * 1e3f + 0.5f); return GPUMPI_SUCCESS;
    default: return GPUMPI_ERR_ARG;
    }
}

int gpumpi_set_tuned_table(gpumpi_world* w, const int8_t* table, size_t bytes) {
    // device layout [3 kinds][3 datatype classes][2 alignment classes][32][16]; kinds 0 Allreduce,
    // 1 Reduce, 2 Alltoall(v); datatype classes 0 float, 1 double / long double, 2 the rest; alignment
    // class 0: every member's buffers 16-byte aligned, 1: not.  A table without datatype classes
    // ([3][2][32][16]) serves every datatype; one without either class ([2 or 3][32][16]) serves both
    // alignments as well; a two-kind table leaves kind 2 unset.
    constexpr size_t cell = 32 * 16;
    constexpr int D = 3, C = 2;
    if (!w || !table || (bytes != 2 * cell && bytes != 3 * cell && bytes != 3 * C * cell && bytes != 3 * D * C * cell))
        return GPUMPI_ERR_ARG;
    std::vector<int8_t> img(3 * D * C * cell, (int8_t)-1);
    if (bytes == 3 * D * C * cell) {
        memcpy(img.data(), table, bytes);
    } else {
        const bool classes = bytes == 3 * C * cell;
        const size_t kinds = classes ? 3 : bytes / cell;
        for (size_t k = 0; k < kinds; k++)
            for (int d = 0; d < D; d++)
                for (int c = 0; c < C; c++)
                    memcpy(img.data() + ((k * D + d) * C + c) * cell, table + (classes ? k * C + c : k) * cell, cell);
    }
    cudaSetDevice(w->device);
    w->h_rt.sel_epoch++;
    if (!w->d_table) CK(cudaMalloc(&w->d_table, img.size()));
    CK(cudaMemcpy(w->d_table, img.data(), img.size(), cudaMemcpyHostToDevice));
    return GPUMPI_SUCCESS;
}

int gpumpi_set_mlp(gpumpi_world* w, const float* params, size_t count) {
    if (!w || !params || count != GPUMPI_MLP_NPARAMS) return GPUMPI_ERR_ARG;
    cudaSetDevice(w->device);
    w->h_rt.sel_epoch++;
    if (!w->d_mlp) CK(cudaMalloc(&w->d_mlp, sizeof(float) * count));
    CK(cudaMemcpy(w->d_mlp, params, sizeof(float) * count, cudaMemcpyHostToDevice));
    return GPUMPI_SUCCESS;
}

int gpumpi_read_trace(gpumpi_world* w, void* host_out, size_t cap, size_t* nout) {
    if (!w || !nout) return GPUMPI_ERR_ARG;
    unsigned long long cnt = 0;
    CK(cudaMemcpy(&cnt, w->h_rt.trace_count, sizeof(cnt), cudaMemcpyDeviceToHost));
    size_t n = std::min<size_t>({(size_t)cnt, cap, (size_t)std::max(0, w->cfg.trace_capacity)});
    if (n && host_out) CK(cudaMemcpy(host_out, w->h_rt.trace, n * sizeof(gpumpi::TraceRec), cudaMemcpyDeviceToHost));
    *nout = n;
    return GPUMPI_SUCCESS;
}

double gpumpi_last_kernel_ms(gpumpi_world* w) { return w ? w->last_ms : 0.0; }

// Picks the block size and engine count for program `pe` (largest of 256/128/64 threads whose
// occupancy co-hosts all ranks, unless the configuration fixes it).
// Dynamic shared memory for T-thread blocks when `bps` blocks share an SM: what is left of the SM's
// shared memory after each block's static allocation and the per-block reservation, capped at the
// 48 KiB that needs no opt-in.  Used for the STAGED fold's TMA stages.
static size_t dyn_smem_for(gpumpi_world* w, const gpumpi_prog_entry* pe, int bps) {
    // without dynamic shared memory the STAGED variants run as DIRECT: no bulk asynchronous copy is
    // pointed at host memory
    if (w->host_aliased) return 0;
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, w->device);
    cudaFuncAttributes fa;
    if (pe->attributes(&fa) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    long long per = (long long)smem_sm / (bps > 0 ? bps : 1) - (long long)fa.sharedSizeBytes - 1024;
    if (per > 48 * 1024) per = 48 * 1024;
    if (w->dyn_smem_cap >= 0 && per > w->dyn_smem_cap) per = w->dyn_smem_cap;
    per &= ~127LL;
    return per >= 4096 ? (size_t)per : 0;
}

static int choose_geometry(gpumpi_world* w, const gpumpi_prog_entry* pe) {
    const int n = w->cfg.nranks;
    int cands[3] = {256, 128, 64};
    int chosen = 0, bps = 0;
    size_t dyn = 0;
    for (int k = 0; k < 3 && !chosen; k++) {
        int T = cands[k];
        if (w->cfg.threads_per_block > 0 && T != w->cfg.threads_per_block) continue;
        int b = 0;
        CK(pe->occupancy(&b, T, 0));  // register-limited occupancy
        if ((long long)b * w->sm_count < n) continue;
        // keep that occupancy and give each block the shared memory that is left over
        size_t d = dyn_smem_for(w, pe, b);
        int b2 = 0;
        CK(pe->occupancy(&b2, T, d));
        while (d > 0 && b2 < b) {
            d = d > 4096 + 1024 ? d - 1024 : 0;
            CK(pe->occupancy(&b2, T, d));
        }
        chosen = T;
        bps = b2;
        dyn = d;
    }
    if (!chosen && w->cfg.threads_per_block > 0) {
        int b = 0;
        CK(pe->occupancy(&b, w->cfg.threads_per_block, 0));
        if ((long long)b * w->sm_count >= n) {
            chosen = w->cfg.threads_per_block;
            bps = b;
        }
    }
    w->dyn_smem = dyn;
    if (!chosen) {
        int b = 0;
        pe->occupancy(&b, 32, 0);
        w->err = "cannot co-host " + std::to_string(n) + " rank blocks on " + std::to_string(w->sm_count) +
                 " SMs (max " + std::to_string((long long)b * w->sm_count) + " blocks of 32 threads)";
        return GPUMPI_ERR_LAUNCH;
    }
    int cap = bps * w->sm_count;
    int eng = cap - n;
    if (w->cfg.engine_blocks >= 0) eng = std::min(eng, w->cfg.engine_blocks);
    w->T = chosen;
    w->blocks_per_sm = bps;
    w->nengines = std::max(0, eng);
    return GPUMPI_SUCCESS;
}

}  // extern "C"

namespace {

// Sets the runtime image for program pe (geometry and policy of the world as it is now).
int prepare_runtime(gpumpi_world* w, const gpumpi_prog_entry* pe) {
    int rc = choose_geometry(w, pe);
    if (rc) return rc;
    Runtime& r = w->h_rt;
    r.T = w->T;
    r.nengines = w->nengines;
    r.variant_override = w->variant_override;
    r.selector_mode = w->selector_mode;
    r.tuned_table = w->d_table;
    r.mlp_params = w->d_mlp;
    r.dyn_smem = (int)w->dyn_smem;
    r.tune_vec = w->tune_vec;
    r.tune_group = w->tune_group;
    return GPUMPI_SUCCESS;
}

// Turns one launch's error records (nb blocks) and the ranks' exit codes into the call's status.
int scan_results(gpumpi_world* w, const gpumpi::ErrorRecord* errs, int nb, const int* exits) {
    int timeout = 0;
    for (int b = 0; b < nb; b++) {
        const gpumpi::ErrorRecord& e = errs[b];
        if (e.code) {
            char buf[256];
            snprintf(buf, sizeof buf, "rank %d: MPI error %d (detail %d) at runtime line %d, info %lld", e.rank,
                     e.code, e.detail, e.line, e.info);
            if (w->err.empty() || e.detail == GPUMPI_ERR_TIMEOUT) w->err = buf;
            if (e.detail == GPUMPI_ERR_TIMEOUT) timeout = 1;
        }
    }
    if (timeout) return GPUMPI_ERR_TIMEOUT;
    for (int i = 0; i < w->cfg.nranks; i++)
        if (exits[i] != 0) {
            w->err = "rank " + std::to_string(i) + " returned " + std::to_string(exits[i]);
            return exits[i];
        }
    return GPUMPI_SUCCESS;
}

// Reads the device error records and exit codes after a finished launch.  Error records describe what
// went wrong inside MPI calls; the calls also returned the codes to the program, so only a run that hit a
// bounded-wait timeout fails here (other errors surface through the ranks' exit codes).
int collect_results(gpumpi_world* w) {
    const Runtime& r = w->h_rt;
    const int nb = w->cfg.nranks + w->nengines;
    CK(cudaMemcpy(w->h_err.data(), r.errors, sizeof(gpumpi::ErrorRecord) * nb, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(w->h_exit.data(), r.exit_codes, sizeof(int) * w->cfg.nranks, cudaMemcpyDeviceToHost));
    return scan_results(w, w->h_err.data(), nb, w->h_exit.data());
}

}  // namespace

extern "C" {

int gpumpi_run_program(gpumpi_world* w, int program, const gpumpi_params* params, void* stream_v, int sync) {
    if (!w || !params) return GPUMPI_ERR_ARG;
    w->err.clear();
    const gpumpi_prog_entry* pe = find_program(program);
    if (!pe) {
        w->err = "unknown program " + std::to_string(program);
        return GPUMPI_ERR_ARG;
    }
    CK(cudaSetDevice(w->device));
    int rc = prepare_runtime(w, pe);
    if (rc) return rc;
    cudaStream_t s = stream_v ? (cudaStream_t)stream_v : w->stream;
    Runtime& r = w->h_rt;
    CK(cudaMemsetAsync(w->d_ctrl, 0, w->ctrl_bytes, s));
    CK(cudaMemcpyAsync(w->d_fixed, &w->h_fixed, sizeof(FixedImage), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(w->d_rt, &r, sizeof(Runtime), cudaMemcpyHostToDevice, s));
    CK(gpumpi_internal_install(w->d_rt, &w->d_fixed->world, &w->d_fixed->gworld, &w->d_fixed->gempty, s));
    CK(cudaEventRecord(w->ev0, s));
    cudaError_t le = pe->launch(w->cfg.nranks + w->nengines, w->T, w->dyn_smem, s, params);
    if (le != cudaSuccess) {
        w->err = std::string("launch of ") + pe->name + ": " + cudaGetErrorString(le);
        cudaGetLastError();
        return GPUMPI_ERR_LAUNCH;
    }
    g_launches++;
    CK(cudaEventRecord(w->ev1, s));
    if (!sync) return GPUMPI_SUCCESS;
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    w->last_ms = ms;
    return collect_results(w);
}

}  // extern "C"

// A recorded launch: the per-launch reset, the runtime install and the cooperative kernel launch of one
// program, captured once and replayed with cudaGraphLaunch.  The reset and install copy from device
// images made at creation, so a replay reads no host memory.
struct gpumpi_graph {
    gpumpi_world* w = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Runtime* d_rt_img = nullptr;
    FixedImage* d_fixed_img = nullptr;
    void** d_install = nullptr;
};

extern "C" {

int gpumpi_graph_create(gpumpi_world* w, int program, const gpumpi_params* params, gpumpi_graph** out) {
    if (!w || !params || !out) return GPUMPI_ERR_ARG;
    *out = nullptr;
    w->err.clear();
    const gpumpi_prog_entry* pe = find_program(program);
    if (!pe) {
        w->err = "unknown program " + std::to_string(program);
        return GPUMPI_ERR_ARG;
    }
    CK(cudaSetDevice(w->device));
    int rc = prepare_runtime(w, pe);
    if (rc) return rc;
    gpumpi_graph* g = new gpumpi_graph();
    g->w = w;
    auto fail = [&](cudaError_t e, const char* what) {
        w->err = std::string(what) + ": " + cudaGetErrorString(e);
        cudaGetLastError();
        gpumpi_graph_destroy(g);
        return GPUMPI_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&g->d_rt_img, sizeof(Runtime)))) return fail(e, "cudaMalloc");
    if ((e = cudaMalloc(&g->d_fixed_img, sizeof(FixedImage)))) return fail(e, "cudaMalloc");
    if ((e = cudaMalloc(&g->d_install, 4 * sizeof(void*)))) return fail(e, "cudaMalloc");
    void* vals[4] = {(void*)w->d_rt, (void*)&w->d_fixed->world, (void*)&w->d_fixed->gworld, (void*)&w->d_fixed->gempty};
    if ((e = cudaMemcpy(g->d_rt_img, &w->h_rt, sizeof(Runtime), cudaMemcpyHostToDevice))) return fail(e, "image");
    if ((e = cudaMemcpy(g->d_fixed_img, &w->h_fixed, sizeof(FixedImage), cudaMemcpyHostToDevice)))
        return fail(e, "image");
    if ((e = cudaMemcpy(g->d_install, vals, sizeof(vals), cudaMemcpyHostToDevice))) return fail(e, "image");
    cudaStream_t cs = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking))) return fail(e, "cudaStreamCreate");
    if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal))) {
        cudaStreamDestroy(cs);
        return fail(e, "cudaStreamBeginCapture");
    }
    cudaError_t ce = cudaMemsetAsync(w->d_ctrl, 0, w->ctrl_bytes, cs);
    if (!ce) ce = cudaMemcpyAsync(w->d_fixed, g->d_fixed_img, sizeof(FixedImage), cudaMemcpyDeviceToDevice, cs);
    if (!ce) ce = cudaMemcpyAsync(w->d_rt, g->d_rt_img, sizeof(Runtime), cudaMemcpyDeviceToDevice, cs);
    if (!ce) ce = gpumpi_internal_install_dev(w->d_rt, g->d_install, cs);
    if (!ce) ce = pe->launch(w->cfg.nranks + w->nengines, w->T, w->dyn_smem, cs, params);
    e = cudaStreamEndCapture(cs, &g->graph);
    cudaStreamDestroy(cs);
    if (ce) return fail(ce, "capture");
    if (e) return fail(e, "cudaStreamEndCapture");
    if ((e = cudaGraphInstantiate(&g->exec, g->graph, 0))) return fail(e, "cudaGraphInstantiate");
    *out = g;
    return GPUMPI_SUCCESS;
}

int gpumpi_graph_launch(gpumpi_graph* g, void* stream_v, int sync) {
    if (!g || !g->exec) return GPUMPI_ERR_ARG;
    gpumpi_world* w = g->w;
    w->err.clear();
    CK(cudaSetDevice(w->device));
    cudaStream_t s = stream_v ? (cudaStream_t)stream_v : w->stream;
    CK(cudaEventRecord(w->ev0, s));
    CK(cudaGraphLaunch(g->exec, s));
    g_launches++;
    CK(cudaEventRecord(w->ev1, s));
    if (!sync) return GPUMPI_SUCCESS;
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    w->last_ms = ms;
    return collect_results(w);
}

int gpumpi_graph_destroy(gpumpi_graph* g) {
    if (!g) return GPUMPI_SUCCESS;
    if (g->w) cudaSetDevice(g->w->device);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->d_rt_img);
    cudaFree(g->d_fixed_img);
    cudaFree(g->d_install);
    delete g;
    return GPUMPI_SUCCESS;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// host-buffer staging and the hot-path entry points
// ------------------------------------------------------------------------------------------------
namespace {

bool is_device_ptr(const void* p) {
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device address of page-locked host memory p (registered or allocated by CUDA), or nullptr.
void* pinned_alias(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// device buffer for slot k holding `bytes`; copies host data in when `in` is non-null
int stage(gpumpi_world* w, int k, const void* host, size_t bytes, bool copy_in, cudaStream_t s, void** dev) {
    if (w->stage_bytes[k] < bytes) {
        cudaFree(w->d_stage[k]);
        w->d_stage[k] = nullptr;
        w->stage_bytes[k] = 0;
        CK(cudaMalloc(&w->d_stage[k], bytes));
        w->stage_bytes[k] = bytes;
    }
    if (copy_in && host && bytes) CK(cudaMemcpyAsync(w->d_stage[k], host, bytes, cudaMemcpyHostToDevice, s));
    *dev = w->d_stage[k];
    return GPUMPI_SUCCESS;
}

struct Buf {
    const void* user;
    size_t bytes;
    bool in, out;
    void* dev;
    bool staged;
};

int run_with_buffers(gpumpi_world* w, int program, gpumpi_params& prm, Buf* bufs, int nbufs, int iters,
                     uint64_t* iter_ns, void* stream_v) {
    cudaStream_t s = stream_v ? (cudaStream_t)stream_v : w->stream;
    struct AliasScope {  // the flag holds for this call only, whatever path returns
        gpumpi_world* w;
        ~AliasScope() { w->host_aliased = false; }
    } alias_scope{w};
    w->host_aliased = false;
    CK(cudaSetDevice(w->device));
    for (int k = 0; k < nbufs; k++) {
        Buf& b = bufs[k];
        b.staged = false;
        b.dev = (void*)b.user;
        if (b.user == (const void*)(intptr_t)1) {  // MPI_IN_PLACE: a marker, not a buffer
            continue;
        }
        if (b.user && !is_device_ptr(b.user)) {
            if (w->host_direct) {
                if (void* alias = pinned_alias(b.user)) {
                    b.dev = alias;
                    w->host_aliased = true;
                    continue;
                }
            }
            int rc = stage(w, k, b.user, b.bytes, b.in, s, &b.dev);
            if (rc) return rc;
            b.staged = true;
        }
    }
    uint64_t* d_ns = nullptr;
    if (iter_ns && iters > 0) {
        void* d;
        int rc = stage(w, 7, nullptr, sizeof(uint64_t) * iters, false, s, &d);
        if (rc) return rc;
        d_ns = (uint64_t*)d;
    }
    for (int k = 0; k < nbufs; k++) prm.p[k] = bufs[k].dev;
    prm.p[6] = d_ns;
    int rc = gpumpi_run_program(w, program, &prm, s, 1);
    for (int k = 0; k < nbufs; k++)
        if (bufs[k].staged && bufs[k].out) CK(cudaMemcpyAsync((void*)bufs[k].user, bufs[k].dev, bufs[k].bytes, cudaMemcpyDeviceToHost, s));
    if (d_ns) CK(cudaMemcpyAsync(iter_ns, d_ns, sizeof(uint64_t) * iters, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return rc;
}

size_t type_bytes(int dt) {
    static const int sizes[GPUMPI_NUM_PREDEFINED_TYPES] = {1, 2, 4, 8, 8, 8, 1, 1, 2, 4, 8, 8, 4, 8, 8, 4, 1, 1,
                                                           2, 4, 8, 1, 2, 4, 8, 8, 8, 16, 16, 1, 8, 8, 16, 16, 8, 16};
    return (dt >= 0 && dt < GPUMPI_NUM_PREDEFINED_TYPES) ? (size_t)sizes[dt] : 0;
}

static_assert(sizeof(gpumpi::ErrorRecord) % sizeof(int) == 0, "records are gathered as ints");

// One launch's error records and exit codes, copied into slot `dst` on the launch's stream (no copy engine
// between the slices' launches: their copies of user data keep the engines busy).
__global__ void gather_records(const int* __restrict__ errs, int nerr, const int* __restrict__ exits, int nexit,
                               int* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nerr + nexit; i += gridDim.x * blockDim.x)
        dst[i] = i < nerr ? errs[i] : exits[i - nerr];
}

// Allreduce between host buffers (rows of `count` elements, one per rank, `per` bytes apart), cut into
// column slices: the same element range of every rank.  Slice j's inputs cross the host link while slice
// j-1 is folded and slice j-2's results cross back, so both directions of the link carry data at once
// (one launch over whole rows moves all inputs, then all results).  Each slice is one launch of the
// collective over the slice's columns with the caller's row stride: every element gets the same fold (the
// canonical rank order, or the variant the policy picks) as in one launch over whole rows.
//   mode 2: inputs and results cross by 2D copies through device staging buffers;
//   mode 3: the kernel reads page-locked inputs in place, results cross by 2D copies;
//   mode 4: inputs cross by 2D copies, the kernel writes page-locked results in place.
// Returns -1 when the call does not qualify (the caller takes the one-launch path).
int allreduce_host_sliced(gpumpi_world* w, const void* sb, void* rb, long long count, int dt, int op,
                          void* stream_v) {
    const int n = w->cfg.nranks;
    const size_t esz = type_bytes(dt);
    const size_t per = (size_t)count * esz;
    // slice width: by default 256 MiB per slice over all ranks and at least 128 KiB per rank (narrower 2D
    // copies lose the two-way overlap); a multiple of 256 bytes per rank (keeps every slice's rows 16-byte
    // aligned when the rows are), at most 64 slices
    size_t sbytes = w->host_slice_bytes > 0 ? (size_t)w->host_slice_bytes
                                            : std::max((size_t)128 << 10, ((size_t)256 << 20) / (size_t)n);
    sbytes = std::max(align_up(sbytes, 256), align_up((per + 63) / 64, 256));
    const long long selems = (long long)(sbytes / esz);
    const int slices = (int)((count + selems - 1) / selems);
    if (slices < 2 || per % 16 != 0) return -1;
    const int mode = w->host_direct;
    void* in_alias = mode == 3 ? pinned_alias(sb) : nullptr;
    void* out_alias = mode == 4 ? pinned_alias(rb) : nullptr;

    cudaStream_t s = stream_v ? (cudaStream_t)stream_v : w->stream;
    CK(cudaSetDevice(w->device));
    // each slice's 2D copy in each direction is split into P row groups on P streams: 2D copies of short
    // rows run at a fraction of the link on one stream
    const int P = std::min(w->host_streams, n);
    for (int k = 0; k < P; k++) {
        if (!w->xs_in[k]) CK(cudaStreamCreateWithFlags(&w->xs_in[k], cudaStreamNonBlocking));
        if (!w->xs_out[k]) CK(cudaStreamCreateWithFlags(&w->xs_out[k], cudaStreamNonBlocking));
    }
    for (auto& e : w->xev)
        if (!e) CK(cudaEventCreate(&e));
    cudaEvent_t ev_in = w->xev[0], ev_fold = w->xev[1], ev_a = w->xev[2], ev_b = w->xev[3];

    struct AliasScope {
        gpumpi_world* w;
        ~AliasScope() { w->host_aliased = false; }
    } alias_scope{w};
    w->host_aliased = in_alias || out_alias;  // no bulk asynchronous copy is pointed at host memory
    const size_t all = per * (size_t)n;
    void *dsend = in_alias, *drecv = out_alias, *drec = nullptr;
    int rc;
    if (!in_alias && (rc = stage(w, 0, nullptr, all, false, s, &dsend))) return rc;
    if (!out_alias && (rc = stage(w, 1, nullptr, all, false, s, &drecv))) return rc;
    const Runtime& r = w->h_rt;
    const int nb = (int)w->h_err.size();  // records of every block the world can launch
    const int nerr = (int)(sizeof(gpumpi::ErrorRecord) / sizeof(int)) * nb;
    const int rec_ints = nerr + n;
    if ((rc = stage(w, 6, nullptr, sizeof(int) * (size_t)rec_ints * slices, false, s, &drec))) return rc;

    // copies wait for whatever the caller queued on its stream before this call (an event's wait refers
    // to its record at the time of the wait call, so one event serves every record-wait pair below)
    CK(cudaEventRecord(ev_a, s));
    for (int k = 0; k < P; k++) CK(cudaStreamWaitEvent(w->xs_in[k], ev_a, 0));
    w->err.clear();
    int launch_rc = GPUMPI_SUCCESS;
    for (int j = 0; j < slices; j++) {
        const long long c0 = (long long)j * selems;
        const long long cn = std::min(selems, count - c0);
        const size_t off = (size_t)c0 * esz, width = (size_t)cn * esz;
        if (!in_alias) {
            for (int k = 0; k < P; k++) {
                const size_t r0 = (size_t)n * k / P, r1 = (size_t)n * (k + 1) / P;
                CK(cudaMemcpy2DAsync((char*)dsend + r0 * per + off, per, (const char*)sb + r0 * per + off, per,
                                     width, r1 - r0, cudaMemcpyHostToDevice, w->xs_in[k]));
                CK(cudaEventRecord(ev_in, w->xs_in[k]));
                CK(cudaStreamWaitEvent(s, ev_in, 0));
            }
        }
        gpumpi_params prm;
        memset(&prm, 0, sizeof(prm));
        prm.i[0] = GPUMPI_COLL_ALLREDUCE;
        prm.i[1] = cn;
        prm.i[2] = dt;
        prm.i[3] = op;
        prm.i[5] = 1;
        prm.i[6] = (long long)per;
        prm.i[7] = (long long)per;
        prm.p[0] = (char*)dsend + off;
        prm.p[1] = (char*)drecv + off;
        launch_rc = gpumpi_run_program(w, GPUMPI_P_COLL, &prm, s, 0);
        if (launch_rc) break;
        gather_records<<<8, 256, 0, s>>>((const int*)r.errors, nerr, r.exit_codes, n, (int*)drec + (size_t)j * rec_ints);
        CK(cudaGetLastError());
        g_launches++;
        if (!out_alias) {
            CK(cudaEventRecord(ev_fold, s));
            for (int k = 0; k < P; k++) {
                const size_t r0 = (size_t)n * k / P, r1 = (size_t)n * (k + 1) / P;
                CK(cudaStreamWaitEvent(w->xs_out[k], ev_fold, 0));
                CK(cudaMemcpy2DAsync((char*)rb + r0 * per + off, per, (const char*)drecv + r0 * per + off, per,
                                     width, r1 - r0, cudaMemcpyDeviceToHost, w->xs_out[k]));
            }
        }
    }
    // the call ends on the caller's stream after the last results have crossed
    for (int k = 0; k < P; k++) {
        CK(cudaEventRecord(ev_fold, w->xs_out[k]));
        CK(cudaStreamWaitEvent(s, ev_fold, 0));
    }
    CK(cudaEventRecord(ev_b, s));
    CK(cudaStreamSynchronize(s));
    for (int k = 0; k < P; k++) CK(cudaStreamSynchronize(w->xs_in[k]));  // inputs in flight when a launch failed
    if (launch_rc) return launch_rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_a, ev_b);
    w->last_ms = ms;
    std::vector<int> rec((size_t)rec_ints * slices);
    CK(cudaMemcpy(rec.data(), drec, sizeof(int) * rec.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < slices; j++) {
        const int* base = rec.data() + (size_t)j * rec_ints;
        rc = scan_results(w, reinterpret_cast<const gpumpi::ErrorRecord*>(base), nb, base + nerr);
        if (rc) return rc;
    }
    return GPUMPI_SUCCESS;
}

int coll_call(gpumpi_world* w, int kind, const void* sb, size_t sbytes, long long sstride, void* rb, size_t rbytes,
              long long rstride, long long count, int dt, int op, int root, int iters, uint64_t* iter_ns,
              void* stream, const int* mats[4], size_t mat_bytes) {
    if (!w) return GPUMPI_ERR_ARG;
    if (!type_bytes(dt)) {
        w->err = "unsupported datatype for the host entry points";
        return GPUMPI_ERR_TYPE;
    }
    gpumpi_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.i[0] = kind;
    prm.i[1] = count;
    prm.i[2] = dt;
    prm.i[3] = op;
    prm.i[4] = root;
    prm.i[5] = iters;
    prm.i[6] = sstride;
    prm.i[7] = rstride;
    // a staged receive buffer is copied in too unless the call writes every byte of it (Allreduce):
    // bytes a collective leaves alone (zero counts, gaps between displacements, non-root ranks) keep
    // the caller's values
    const bool writes_all = kind == GPUMPI_COLL_ALLREDUCE && sb != (const void*)(intptr_t)1 && rstride > 0 &&
                            (size_t)rstride * w->cfg.nranks == rbytes;
    Buf b[6] = {{sb, sbytes, true, false, nullptr, false},
                {rb, rbytes, !writes_all, true, nullptr, false},
                {mats ? mats[0] : nullptr, mat_bytes, true, false, nullptr, false},
                {mats ? mats[1] : nullptr, mat_bytes, true, false, nullptr, false},
                {mats ? mats[2] : nullptr, mat_bytes, true, false, nullptr, false},
                {mats ? mats[3] : nullptr, mat_bytes, true, false, nullptr, false}};
    if (kind == GPUMPI_COLL_ALLREDUCE && w->host_direct >= 2 && iters == 1 && !iter_ns && sb && rb &&
        sb != (const void*)(intptr_t)1 && sstride == rstride && (size_t)sstride == (size_t)count * type_bytes(dt) &&
        !is_device_ptr(sb) && !is_device_ptr(rb)) {
        int rc = allreduce_host_sliced(w, sb, rb, count, dt, op, stream);
        if (rc >= 0) return rc;
    }
    return run_with_buffers(w, GPUMPI_P_COLL, prm, b, 6, iters, iter_ns, stream);
}

}  // namespace

extern "C" {

int gpumpi_test_run(gpumpi_world* w, int test, uint8_t* ok, int64_t* outi, double* outd) {
    if (!w) return GPUMPI_ERR_ARG;
    const int n = w->cfg.nranks;
    gpumpi_params prm;
    memset(&prm, 0, sizeof(prm));
    std::vector<uint8_t> hok(n, 0);
    std::vector<int64_t> hi((size_t)n * 64, 0);
    std::vector<double> hd((size_t)n * 64, 0.0);
    Buf b[3] = {{hok.data(), (size_t)n, true, true, nullptr, false},
                {hi.data(), sizeof(int64_t) * n * 64, true, true, nullptr, false},
                {hd.data(), sizeof(double) * n * 64, true, true, nullptr, false}};
    int rc = run_with_buffers(w, test, prm, b, 3, 0, nullptr, nullptr);
    if (ok) memcpy(ok, hok.data(), n);
    if (outi) memcpy(outi, hi.data(), sizeof(int64_t) * n * 64);
    if (outd) memcpy(outd, hd.data(), sizeof(double) * n * 64);
    return rc;
}

int gpumpi_allreduce(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int dt, int op, int iters,
                     uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    size_t per = (size_t)count * type_bytes(dt);
    size_t all = per * w->cfg.nranks;
    return coll_call(w, GPUMPI_COLL_ALLREDUCE, sendbuf, all, (long long)per, recvbuf, all, (long long)per, count, dt,
                     op, 0, iters, iter_ns, stream, nullptr, 0);
}

int gpumpi_reduce(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int dt, int op, int root,
                  int iters, uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    size_t per = (size_t)count * type_bytes(dt);
    size_t all = per * w->cfg.nranks;
    // recvbuf is rank-major too (only root's slot is written)
    return coll_call(w, GPUMPI_COLL_REDUCE, sendbuf, all, (long long)per, recvbuf, all, (long long)per, count, dt, op,
                     root, iters, iter_ns, stream, nullptr, 0);
}

int gpumpi_bcast(gpumpi_world* w, void* buf, long long count, int dt, int root, int iters, uint64_t* iter_ns,
                 void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    size_t per = (size_t)count * type_bytes(dt);
    size_t all = per * w->cfg.nranks;
    return coll_call(w, GPUMPI_COLL_BCAST, nullptr, 0, 0, buf, all, (long long)per, count, dt, 0, root, iters, iter_ns,
                     stream, nullptr, 0);
}

int gpumpi_alltoall(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long cpp, int dt, int iters,
                    uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    size_t per = (size_t)cpp * type_bytes(dt) * w->cfg.nranks;
    size_t all = per * w->cfg.nranks;
    return coll_call(w, GPUMPI_COLL_ALLTOALL, sendbuf, all, (long long)per, recvbuf, all, (long long)per, cpp, dt, 0,
                     0, iters, iter_ns, stream, nullptr, 0);
}

int gpumpi_allgather(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int dt, int iters,
                     uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    size_t per = (size_t)count * type_bytes(dt);
    return coll_call(w, GPUMPI_COLL_ALLGATHER, sendbuf, per * w->cfg.nranks, (long long)per, recvbuf,
                     per * w->cfg.nranks * w->cfg.nranks, (long long)(per * w->cfg.nranks), count, dt, 0, 0, iters,
                     iter_ns, stream, nullptr, 0);
}

int gpumpi_alltoallv(gpumpi_world* w, const void* sendbuf, long long send_stride, const int* sendcounts,
                     const int* sdispls, void* recvbuf, long long recv_stride, const int* recvcounts, const int* rdispls,
                     int dt, int iters, uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    const int* mats[4] = {sendcounts, sdispls, recvcounts, rdispls};
    size_t n = (size_t)w->cfg.nranks;
    return coll_call(w, GPUMPI_COLL_ALLTOALLV, sendbuf, (size_t)send_stride * n, send_stride, recvbuf,
                     (size_t)recv_stride * n, recv_stride, 0, dt, 0, 0, iters, iter_ns, stream, mats,
                     sizeof(int) * n * n);
}

int gpumpi_pingpong(gpumpi_world* w, void* bufs, long long bytes, int pairs, int iters, int nonblocking,
                    uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    gpumpi_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.i[0] = bytes;
    prm.i[1] = iters;
    prm.i[2] = nonblocking;
    prm.i[3] = pairs;
    prm.i[4] = bytes;
    Buf b[1] = {{bufs, (size_t)bytes * w->cfg.nranks, true, true, nullptr, false}};
    return run_with_buffers(w, GPUMPI_P_PINGPONG, prm, b, 1, iters, iter_ns, stream);
}

int gpumpi_ring(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long bytes, int iters, int nonblocking,
                uint64_t* iter_ns, void* stream) {
    if (!w) return GPUMPI_ERR_ARG;
    gpumpi_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.i[0] = bytes;
    prm.i[1] = iters;
    prm.i[2] = nonblocking;
    prm.i[4] = bytes;
    Buf b[2] = {{sendbuf, (size_t)bytes * w->cfg.nranks, true, false, nullptr, false},
                {recvbuf, (size_t)bytes * w->cfg.nranks, false, true, nullptr, false}};
    return run_with_buffers(w, GPUMPI_P_RING, prm, b, 2, iters, iter_ns, stream);
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// The launcher of a converted program (replaces gpu_libs/gpu_main/main.cu:133-320): the arguments
// before `---gpumpi` are the program's, the ones after configure the run (gpumpi_parse_args); every
// rank runs the program with a device copy of its arguments; the exit status is 1 when the run failed
// or any rank returned non-zero (main.cu:126-129,320), with the reason on stderr.
// ------------------------------------------------------------------------------------------------
extern "C" int gpumpi_main(int argc, char** argv, int program) {
    gpumpi_config cfg;
    gpumpi_config_init(&cfg);
    const int pos = gpumpi_parse_args(argc, argv, &cfg);
    const int pargc = pos < 0 ? argc : pos;
    gpumpi_world* w = nullptr;
    int rc = gpumpi_world_create(&cfg, &w);
    if (rc) {
        fprintf(stderr, "gpumpi: %s\n", gpumpi_last_error(nullptr));
        return 1;
    }
    // argv on the device: pointer table, then the strings
    size_t bytes = sizeof(char*) * (size_t)(pargc + 1);
    for (int i = 0; i < pargc; i++) bytes += strlen(argv[i]) + 1;
    std::vector<char> img(bytes, 0);
    char* d_img = nullptr;
    if (cudaMalloc(&d_img, bytes) != cudaSuccess) {
        fprintf(stderr, "gpumpi: cudaMalloc of %zu bytes for the arguments failed\n", bytes);
        gpumpi_world_destroy(w);
        return 1;
    }
    char** tab = (char**)img.data();
    size_t off = sizeof(char*) * (size_t)(pargc + 1);
    for (int i = 0; i < pargc; i++) {
        const size_t len = strlen(argv[i]) + 1;
        memcpy(img.data() + off, argv[i], len);
        tab[i] = d_img + off;
        off += len;
    }
    tab[pargc] = nullptr;
    gpumpi_params prm;
    memset(&prm, 0, sizeof(prm));
    prm.i[0] = pargc;
    prm.p[0] = d_img;
    if (cudaMemcpy(d_img, img.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = GPUMPI_ERR_CUDA;
    else rc = gpumpi_run_program(w, program, &prm, nullptr, 1);
    if (rc) fprintf(stderr, "gpumpi: %s\n", gpumpi_last_error(w));
    cudaFree(d_img);
    gpumpi_world_destroy(w);
    return rc ? 1 : 0;
}
