// Native serving pool (tvbg_serve_*): continuous batching of sweep requests
// on the lane-interleaved group kernel.
//
// A request is copied in at tvbg_serve_admit and planned on the host the way
// tvb_hpc.groups.GroupSet plans it: integer delays per distinct speed
// (tvbg_delays), per delay table the block length K (8 or 4, K <= d_min + 1)
// and ring length nh (a power of two >= d_max + 1 + K, >= 8), edges packed
// per table, nodes visited by in-degree (descending, stable), instances in
// groups of eight per table (request-local index = Philox key word 1), one
// CTA or cluster per group (the smallest cluster whose CTAs stay within
// 1024 threads).  Its device buffers are one allocation made when the
// request is admitted: when its footprint fits the budget and the device.
//
// A tick uploads every active request's group records for its next chunk
// (t0, steps per lane) and launches its groups -- one launch per block
// length -- on the request's own stream; the streams join the pool's
// stream, the pool waits, checks each request's device status word, and
// retires finished requests (state gathered from the lanes to the host,
// device memory freed).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "tvbg_abi_internal.h"
#include "tvbg_group_launch.cuh"

using namespace tvbg;

namespace {
struct Request;
}

struct tvbg_serve {
    int64_t cap = 0;               // budget at creation: a request larger never fits
    int64_t budget = 0, used = 0;  // current admission budget (tvbg_serve_set_budget)
    int32_t chunk = 0;
    int64_t cta_cap = 0;           // admission stops at this many resident CTAs (0: no cap,
                                   // -1: 3 x SMs)
    int64_t active_ctas = 0;
    int64_t next_id = 1;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::map<int64_t, Request*> all;
    std::vector<int64_t> finished;                 // retired ids not yet fetched
    std::map<size_t, std::vector<void*>> pinned;   // free pinned staging blocks by size
    // chunk completions, counted by a host function after each chunk; a
    // tick with nothing completed waits on cv for the next one
    std::mutex mu;
    std::condition_variable cv;
    uint64_t completions = 0;
};

namespace {

constexpr int L = TVBG_GROUP_LANES;

// Pinned host staging, recycled through the pool (cudaFreeHost would wait
// for the device): blocks of a power of two >= 256 bytes.
size_t pinned_class(size_t n) {
    size_t c = 256;
    while (c < n) c <<= 1;
    return c;
}
void* pinned_get(tvbg_serve& p, size_t bytes) {
    std::vector<void*>& v = p.pinned[bytes];
    if (!v.empty()) {
        void* h = v.back();
        v.pop_back();
        return h;
    }
    void* h = nullptr;
    return cudaMallocHost(&h, bytes) == cudaSuccess ? h : nullptr;
}
void pinned_put(tvbg_serve& p, void* h, size_t bytes) {
    if (h) p.pinned[bytes].push_back(h);
}

// Host function enqueued after each chunk: counts it and wakes a waiting tick.
void CUDART_CB chunk_done(void* arg) {
    tvbg_serve* p = static_cast<tvbg_serve*>(arg);
    {
        std::lock_guard<std::mutex> lk(p->mu);
        ++p->completions;
    }
    p->cv.notify_all();
}

// (state variables, per-node parameters, observables) of each model id
struct ModelShape {
    int ns, np, nobs;
};
bool model_shape(int model, ModelShape* s) {
    switch (model) {
        case TVBG_MODEL_KURAMOTO: *s = {1, 1, 2}; return true;
        case TVBG_MODEL_G2DO: *s = {2, 1, 2}; return true;
        case TVBG_MODEL_MPR: *s = {2, 1, 2}; return true;
        case TVBG_MODEL_LINEAR: *s = {1, 1, 1}; return true;
        case TVBG_MODEL_G2DOSC: *s = {2, 1, 2}; return true;
        case TVBG_MODEL_RWW: *s = {1, 2, 1}; return true;
        case TVBG_MODEL_JANSENRIT: *s = {6, 2, 1}; return true;
        default: return false;
    }
}

size_t align_up(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

__global__ void fill_cos_channel(float* ring, long long n) {
    // [..][2][L] layout: channel 1 (cos) of every slot holds cos 0 = 1
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        ring[i] = ((i / L) & 1) ? 1.0f : 0.0f;
}

struct Request {
    int64_t id = 0;
    int status = TVBG_SERVE_QUEUED;
    // inputs
    int model = 0, cfun = 0, N = 0, nnz = 0, n_inst = 0, npar = 0;
    ModelShape shape{};
    int64_t nsteps = 0, done = 0;
    float dt = 0.0f;
    uint64_t seed = 0;
    uint32_t flags = 0;
    float cf_b = 0.0f, cf_p[3] = {0, 0, 0}, sigma[4] = {0, 0, 0, 0}, consts[16] = {};
    std::vector<float> couplings, state0, nparam;
    // plan
    int channels = 1, threads = 0, cluster = 1, tpn = 1;  // tpn 2: pipelined group kernel
    std::vector<int32_t> row, nodes;
    std::vector<float> wsum;
    std::vector<tvbg_edge> edges;     // [tables][nnz]
    std::vector<int> table_k, table_lognh, table_dmin;
    std::vector<int> g_table;         // per group
    std::vector<std::vector<int>> members;
    size_t off_edges = 0, off_row = 0, off_wsum = 0, off_nodes = 0, off_ring = 0, off_state = 0,
           off_nparam = 0, off_groups = 0, off_order = 0, off_status = 0, bytes = 0;
    std::vector<size_t> ring_off;     // per group, floats from off_ring
    std::vector<int32_t> order;       // per block length, the groups of that length
    std::vector<int> k_list, k_start, k_count;
    // device
    char* dev = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done_ev = nullptr;
    std::vector<tvbg_group> records;
    tvbg_group* h_records = nullptr;  // pinned staging of records (asynchronous uploads)
    size_t h_records_bytes = 0;       // its block size (pool cache class)
    int32_t* h_status = nullptr;      // pinned copy of the status word, read once its chunk is done
    int64_t inflight = 0;             // steps of the chunk running now (0: none)
    int64_t ctas = 0;                 // CTAs of one chunk: groups x cluster
    std::vector<float> result;        // [n_inst][N][ns] once done
};

// The plain group kernel's shape: the smallest cluster whose CTAs stay
// within 1024 threads, one node per 8-lane slot (several beyond 8 CTAs).
void plain_shape(Request& r) {
    int c = 1;
    while (L * ((r.N + c - 1) / c) > 1024 && c < 8) c *= 2;
    r.tpn = 1;
    r.cluster = c;
    const int per = (r.N + c - 1) / c;
    r.threads = std::min(1024, 32 * ((L * per + 31) / 32));
}

int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Host plan of a request (no device work); fills the byte layout.
int plan(Request& r, const tvbg_serve_request& q) {
    const int N = r.N, nnz = r.nnz;
    // delay tables, one per distinct speed (sorted, as numpy.unique)
    std::vector<float> speeds(q.speeds, q.speeds + r.n_inst);
    std::vector<float> uniq = speeds;
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    std::vector<int> tab_of(r.n_inst);
    for (int b = 0; b < r.n_inst; ++b)
        tab_of[b] = static_cast<int>(std::lower_bound(uniq.begin(), uniq.end(), speeds[b]) - uniq.begin());
    const int T = static_cast<int>(uniq.size());
    r.edges.resize(static_cast<size_t>(T) * std::max(1, nnz));
    std::vector<int32_t> d(std::max(1, nnz));
    for (int t = 0; t < T; ++t) {
        if (nnz > 0) {
            int rc = tvbg_delays(nnz, q.lengths, uniq[t], q.dt, q.rounding, d.data());
            if (rc) return rc;
        }
        int dmin = 7, dmax = 0;
        if (nnz > 0) {
            dmin = *std::min_element(d.begin(), d.begin() + nnz);
            dmax = *std::max_element(d.begin(), d.begin() + nnz);
        }
        const int k = dmin + 1 >= 8 ? 8 : (dmin + 1 >= 4 ? 4 : 0);
        if (k == 0)
            return set_error(TVBG_EUNSUPPORTED,
                             "tvbg_serve_admit: delays shorter than the group kernel's blocks (d_min < 3)");
        const int nh = std::max(8, next_pow2(dmax + 1 + k));
        int lognh = 0;
        while ((1 << lognh) < nh) ++lognh;
        if (lognh > 16) return set_error(TVBG_EINVAL, "tvbg_serve_admit: delays beyond 2^16 - 9 steps");
        r.table_k.push_back(k);
        r.table_lognh.push_back(lognh);
        r.table_dmin.push_back(dmin);
        if (nnz > 0) {
            int rc = tvbg_pack_edges_group(N, nnz, q.row, q.col, q.weights, d.data(), lognh,
                                           r.edges.data() + static_cast<size_t>(t) * nnz);
            if (rc) return rc;
        }
    }
    // per-node constants: in-edge weight sums and the visiting order
    r.row.assign(q.row, q.row + N + 1);
    r.wsum.assign(N, 0.0f);
    std::vector<int> deg(N);
    for (int i = 0; i < N; ++i) {
        deg[i] = q.row[i + 1] - q.row[i];
        float s = 0.0f;
        for (int e = q.row[i]; e < q.row[i + 1]; ++e) s += q.weights[e];
        r.wsum[i] = s;
    }
    r.nodes.resize(N);
    for (int i = 0; i < N; ++i) r.nodes[i] = i;
    std::stable_sort(r.nodes.begin(), r.nodes.end(), [&](int a, int b) { return deg[a] > deg[b]; });
    // groups: per table, eight instances in index order
    for (int t = 0; t < T; ++t) {
        std::vector<int> idx;
        for (int b = 0; b < r.n_inst; ++b)
            if (tab_of[b] == t) idx.push_back(b);
        for (size_t g0 = 0; g0 < idx.size(); g0 += L) {
            r.members.emplace_back(idx.begin() + g0, idx.begin() + std::min(idx.size(), g0 + L));
            r.g_table.push_back(t);
        }
    }
    const int G = static_cast<int>(r.members.size());
    // launch shape: the pipelined kernel on its smallest cluster that holds
    // one node per slot, where every delay is at least 2K - 1 steps (its
    // results equal the plain kernel's); else the plain kernel on the smallest
    // cluster whose CTAs stay within 1024 threads
    bool pipe = true;
    for (int t = 0; t < T; ++t) pipe = pipe && r.table_dmin[t] >= 2 * r.table_k[t] - 1;
    r.tpn = 1;
    if (pipe) {
        for (int c : {1, 2, 3, 4, 6, 8, 12, 16}) {
            const int thr = 2 * 32 * ((L * ((N + c - 1) / c) + 31) / 32);
            if (thr <= 1024) {
                r.tpn = TVBG_GROUP_PIPELINED;
                r.cluster = c;
                r.threads = thr;
                break;
            }
        }
    }
    if (r.tpn != TVBG_GROUP_PIPELINED) plain_shape(r);
    // launch order: one launch per block length, groups in index order
    for (int k : {4, 8}) {
        int cnt = 0;
        const int start = static_cast<int>(r.order.size());
        for (int g = 0; g < G; ++g)
            if (r.table_k[r.g_table[g]] == k) {
                r.order.push_back(g);
                ++cnt;
            }
        if (cnt) {
            r.k_list.push_back(k);
            r.k_start.push_back(start);
            r.k_count.push_back(cnt);
        }
    }
    // byte layout of the one device allocation
    const int ns = r.shape.ns, np = r.npar, C = r.channels;
    size_t o = 0;
    r.off_edges = o;
    o = align_up(o + r.edges.size() * sizeof(tvbg_edge));
    r.off_row = o;
    o = align_up(o + (N + 1) * sizeof(int32_t));
    r.off_wsum = o;
    o = align_up(o + N * sizeof(float));
    r.off_nodes = o;
    o = align_up(o + N * sizeof(int32_t));
    r.off_ring = o;
    size_t ring_floats = 0;
    for (int g = 0; g < G; ++g) {
        r.ring_off.push_back(ring_floats);
        const size_t R = (static_cast<size_t>(1) << r.table_lognh[r.g_table[g]]) + 8;
        ring_floats += static_cast<size_t>(N) * R * L * C;
    }
    o = align_up(o + ring_floats * sizeof(float));
    r.off_state = o;
    o = align_up(o + static_cast<size_t>(G) * N * ns * L * sizeof(float));
    r.off_nparam = o;
    o = align_up(o + static_cast<size_t>(G) * N * np * L * sizeof(float));
    r.off_groups = o;
    o = align_up(o + static_cast<size_t>(G) * sizeof(tvbg_group));
    r.off_order = o;
    o = align_up(o + std::max<size_t>(1, r.order.size()) * sizeof(int32_t));
    r.off_status = o;
    o = align_up(o + sizeof(int32_t));
    r.bytes = o;
    return TVBG_OK;
}

// Allocate, upload and initialise the request's device state.
// Whether the device can hold one cluster of the pipelined shape of r
// (cudaOccupancyMaxActiveClusters); the plain shape is used where not.
bool pipelined_fits(const Request& r) {
    for (int k : r.k_list) {
        GroupKernel kfn = lookup_group_kernel(r.model, r.cfun, k, true);
        if (!kfn) return false;
        const size_t smem = group_pipelined_smem_bytes(k, r.threads, group_channels(r.cfun));
        if (smem + sizeof(tvbg_group) > 48u * 1024u &&
            cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)) != cudaSuccess)
            return (cudaGetLastError(), false);
        if (r.cluster > 8 &&
            cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
            return (cudaGetLastError(), false);
        cudaLaunchConfig_t lc;
        std::memset(&lc, 0, sizeof(lc));
        lc.gridDim = dim3(static_cast<unsigned>(r.cluster), 1, 1);
        lc.blockDim = dim3(static_cast<unsigned>(r.threads), 1, 1);
        lc.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = static_cast<unsigned>(r.cluster);
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, reinterpret_cast<const void*>(kfn), &lc) != cudaSuccess)
            return (cudaGetLastError(), false);
        if (n < 1) return false;
    }
    return true;
}

// Device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync on the
// request's stream): admitting or retiring a request never waits for the
// other requests' chunks, as cudaFree would.
int materialise(tvbg_serve& p, Request& r) {
    if (r.tpn == TVBG_GROUP_PIPELINED && !pipelined_fits(r)) plain_shape(r);
    cudaError_t e = cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r.done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: stream");
    e = cudaMallocAsync(reinterpret_cast<void**>(&r.dev), r.bytes, r.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);  // usable from any stream
    if (e != cudaSuccess) {
        r.dev = nullptr;
        return set_cuda_error(e, "tvbg_serve: cudaMallocAsync");
    }
    const int N = r.N, ns = r.shape.ns, np = r.npar, G = static_cast<int>(r.members.size());
    r.h_records_bytes = pinned_class(static_cast<size_t>(std::max(1, G)) * sizeof(tvbg_group));
    r.h_records = static_cast<tvbg_group*>(pinned_get(p, r.h_records_bytes));
    r.h_status = static_cast<int32_t*>(pinned_get(p, 256));
    if (!r.h_records || !r.h_status) return set_error(TVBG_ECUDA, "tvbg_serve: pinned staging");
    *r.h_status = 0;
    r.ctas = static_cast<int64_t>(G) * r.cluster;
    // lane-interleaved state and parameters [G][N][*][L]
    std::vector<float> gstate(static_cast<size_t>(G) * N * ns * L, 0.0f);
    std::vector<float> gpar(static_cast<size_t>(G) * N * np * L, 0.0f);
    for (int g = 0; g < G; ++g)
        for (size_t l = 0; l < r.members[g].size(); ++l) {
            const int b = r.members[g][l];
            for (int n = 0; n < N; ++n) {
                for (int v = 0; v < ns; ++v)
                    gstate[((static_cast<size_t>(g) * N + n) * ns + v) * L + l] =
                        r.state0[(static_cast<size_t>(b) * N + n) * ns + v];
                for (int v = 0; v < np; ++v)
                    gpar[((static_cast<size_t>(g) * N + n) * np + v) * L + l] =
                        r.nparam[(static_cast<size_t>(b) * N + n) * np + v];
            }
        }
    struct Up {
        size_t off;
        const void* src;
        size_t n;
    } ups[] = {{r.off_edges, r.edges.data(), r.edges.size() * sizeof(tvbg_edge)},
               {r.off_row, r.row.data(), r.row.size() * sizeof(int32_t)},
               {r.off_wsum, r.wsum.data(), r.wsum.size() * sizeof(float)},
               {r.off_nodes, r.nodes.data(), r.nodes.size() * sizeof(int32_t)},
               {r.off_state, gstate.data(), gstate.size() * sizeof(float)},
               {r.off_nparam, gpar.data(), gpar.size() * sizeof(float)},
               {r.off_order, r.order.data(), r.order.size() * sizeof(int32_t)}};
    for (const Up& u : ups) {
        if (u.n == 0) continue;
        e = cudaMemcpy(r.dev + u.off, u.src, u.n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: upload");
    }
    e = cudaMemset(r.dev + r.off_status, 0, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(r.dev + r.off_ring, 0, r.off_state - r.off_ring);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: memset");
    if (r.channels == 2) {  // zero history of the Kuramoto coupling: (sin 0, cos 0)
        const long long n = static_cast<long long>((r.off_state - r.off_ring) / sizeof(float));
        fill_cos_channel<<<1024, 256, 0, r.stream>>>(reinterpret_cast<float*>(r.dev + r.off_ring), n);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: ring init");
    }
    // group records (t0 and step counts are set per tick)
    r.records.assign(G, tvbg_group{});
    const uint64_t seed = r.seed;
    for (int g = 0; g < G; ++g) {
        tvbg_group& rec = r.records[g];
        const int t = r.g_table[g];
        rec.edges = reinterpret_cast<const tvbg_edge*>(r.dev + r.off_edges) +
                    static_cast<size_t>(t) * std::max(1, r.nnz);
        rec.row = reinterpret_cast<const int32_t*>(r.dev + r.off_row);
        rec.wsum = reinterpret_cast<const float*>(r.dev + r.off_wsum);
        rec.nodes = reinterpret_cast<const int32_t*>(r.dev + r.off_nodes);
        rec.ring = reinterpret_cast<float*>(r.dev + r.off_ring) + r.ring_off[g];
        rec.state = reinterpret_cast<float*>(r.dev + r.off_state) + static_cast<size_t>(g) * N * ns * L;
        rec.nparam = reinterpret_cast<const float*>(r.dev + r.off_nparam) + static_cast<size_t>(g) * N * np * L;
        rec.N = N;
        rec.nnz = r.nnz;
        rec.lognh = r.table_lognh[t];
        rec.model = r.model;
        rec.cfun = r.cfun;
        rec.flags = r.flags;
        rec.trace_every = 1;
        rec.trace_len = 1;
        rec.trace_nobs = r.shape.nobs;
        rec.bold_period = 1;
        rec.bold_len = 0;
        rec.bold_obs = (r.model == TVBG_MODEL_KURAMOTO || r.model == TVBG_MODEL_G2DO) ? 1 : 0;
        rec.dmin = r.table_dmin[t];
        rec.seed_lo = static_cast<uint32_t>(seed & 0xffffffffu);
        rec.seed_hi = static_cast<uint32_t>(seed >> 32);
        rec.dt = r.dt;
        rec.sqrt_dt = std::sqrt(r.dt);
        rec.dt_bold = static_cast<float>(static_cast<double>(r.dt) / 1000.0);
        rec.cf_b = r.cf_b;
        std::memcpy(rec.cf_p, r.cf_p, sizeof(rec.cf_p));
        std::memcpy(rec.sigma, r.sigma, sizeof(rec.sigma));
        std::memcpy(rec.consts, r.consts, sizeof(rec.consts));
        for (size_t l = 0; l < r.members[g].size(); ++l) {
            rec.lanes[l].cf_a = r.couplings[r.members[g][l]];
            rec.lanes[l].inst_id = static_cast<uint32_t>(r.members[g][l]);
        }
    }
    return TVBG_OK;
}

void release(tvbg_serve& p, Request& r) {
    if (r.stream) cudaStreamSynchronize(r.stream);   // this request's chunk only
    if (r.dev) cudaFreeAsync(r.dev, r.stream);
    pinned_put(p, r.h_records, r.h_records_bytes);
    pinned_put(p, r.h_status, 256);
    r.h_records = nullptr;
    r.h_status = nullptr;
    if (r.done_ev) cudaEventDestroy(r.done_ev);
    if (r.stream) cudaStreamDestroy(r.stream);
    r.dev = nullptr;
    r.stream = nullptr;
    r.done_ev = nullptr;
    r.inflight = 0;
    r.records.clear();
    r.records.shrink_to_fit();
}

// Enqueue the next `steps` steps of every group of r on r.stream, then the
// status word's copy, the chunk's event and its completion count.
int launch_chunk(tvbg_serve& p, Request& r, int64_t steps) {
    const int G = static_cast<int>(r.records.size());
    for (int g = 0; g < G; ++g) {
        tvbg_group& rec = r.records[g];
        rec.t0 = r.done;
        rec.nsteps = static_cast<int32_t>(steps);
        for (size_t l = 0; l < r.members[g].size(); ++l) rec.lanes[l].nsteps = static_cast<int32_t>(steps);
    }
    // refilling the pinned staging is safe: a request's next chunk is
    // launched only once its previous chunk's event (after that upload) is done
    std::memcpy(r.h_records, r.records.data(), G * sizeof(tvbg_group));
    cudaError_t e = cudaMemcpyAsync(r.dev + r.off_groups, r.h_records, G * sizeof(tvbg_group),
                                    cudaMemcpyHostToDevice, r.stream);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: group records");
    static const ErrSink sink{set_error, set_cuda_error};
    for (size_t i = 0; i < r.k_list.size(); ++i) {
        tvbg_launch cfg{};
        cfg.model = r.model;
        cfg.cfun = r.cfun;
        cfg.threads = r.threads;
        cfg.cluster = r.cluster;
        cfg.tpn = r.tpn;
        cfg.block_k = r.k_list[i];
        cfg.d_status = reinterpret_cast<int32_t*>(r.dev + r.off_status);
        cfg.d_order = reinterpret_cast<const int32_t*>(r.dev + r.off_order) + r.k_start[i];
        const bool pipe = r.tpn == TVBG_GROUP_PIPELINED;
        GroupKernel k = lookup_group_kernel(r.model, r.cfun, r.k_list[i], pipe);
        if (!k) return set_error(TVBG_EUNSUPPORTED, "tvbg_serve: group kernel not built");
        const size_t smem =
            pipe ? group_pipelined_smem_bytes(cfg.block_k, cfg.threads, group_channels(cfg.cfun))
                 : group_smem_bytes(cfg.block_k, cfg.threads, group_channels(cfg.cfun));
        int rc = launch_group_kernel(k, reinterpret_cast<const tvbg_group*>(r.dev + r.off_groups),
                                     r.k_count[i], &cfg, r.cluster, smem, r.stream, sink);
        if (rc) return rc;
    }
    // the status word comes back with the chunk (read after the tick's sync)
    e = cudaMemcpyAsync(r.h_status, r.dev + r.off_status, sizeof(int32_t), cudaMemcpyDeviceToHost,
                        r.stream);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: status copy");
    e = cudaEventRecord(r.done_ev, r.stream);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(r.stream, chunk_done, &p);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: event");
    r.inflight = steps;
    return TVBG_OK;
}

// Gather the final state [n_inst][N][ns] from the lanes.
int collect(Request& r) {
    const int N = r.N, ns = r.shape.ns, G = static_cast<int>(r.members.size());
    std::vector<float> gstate(static_cast<size_t>(G) * N * ns * L);
    cudaError_t e = cudaMemcpy(gstate.data(), r.dev + r.off_state, gstate.size() * sizeof(float),
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve: state download");
    r.result.assign(static_cast<size_t>(r.n_inst) * N * ns, 0.0f);
    for (int g = 0; g < G; ++g)
        for (size_t l = 0; l < r.members[g].size(); ++l) {
            const int b = r.members[g][l];
            for (int n = 0; n < N; ++n)
                for (int v = 0; v < ns; ++v)
                    r.result[(static_cast<size_t>(b) * N + n) * ns + v] =
                        gstate[((static_cast<size_t>(g) * N + n) * ns + v) * L + l];
        }
    return TVBG_OK;
}

// Launch the next chunk of every active request with none running.
int launch_idle(tvbg_serve& p) {
    for (Request* r : p.active) {
        if (r->inflight || r->done >= r->nsteps) continue;
        int rc = launch_chunk(p, *r, std::min<int64_t>(p.chunk, r->nsteps - r->done));
        if (rc) return rc;
    }
    return TVBG_OK;
}

}  // namespace

extern "C" {

int tvbg_serve_create(int64_t hbm_budget, int32_t chunk, void* stream, tvbg_serve** out) {
    if (!out || hbm_budget <= 0 || chunk <= 0) return set_error(TVBG_EINVAL, "tvbg_serve_create: bad arguments");
    tvbg_serve* p = new (std::nothrow) tvbg_serve;
    if (!p) return set_error(TVBG_EINVAL, "tvbg_serve_create: out of host memory");
    p->budget = hbm_budget;
    p->cap = hbm_budget;
    p->chunk = chunk;
    (void)stream;  // reserved: every request runs on a stream of its own
    *out = p;
    return TVBG_OK;
}

int tvbg_serve_destroy(tvbg_serve* p) {
    if (!p) return TVBG_OK;
    for (auto& kv : p->all) {   // each waits for its request's chunk (and callback)
        release(*p, *kv.second);
        delete kv.second;
    }
    for (auto& kv : p->pinned)
        for (void* h : kv.second) cudaFreeHost(h);
    delete p;
    return TVBG_OK;
}

int tvbg_serve_admit(tvbg_serve* p, const tvbg_serve_request* q, int64_t* id) {
    if (!p || !q || !id) return set_error(TVBG_EINVAL, "tvbg_serve_admit: null");
    ModelShape sh{};
    if (!model_shape(q->model, &sh)) return set_error(TVBG_EUNSUPPORTED, "tvbg_serve_admit: unknown model");
    const bool separable = q->cfun == TVBG_CFUN_LINEAR || q->cfun == TVBG_CFUN_DIFF ||
                           q->cfun == TVBG_CFUN_SIGMOIDAL;
    const bool kuramoto = q->model == TVBG_MODEL_KURAMOTO && q->cfun == TVBG_CFUN_KURAMOTO;
    if (!separable && !kuramoto)
        return set_error(TVBG_EUNSUPPORTED, "tvbg_serve_admit: coupling not on the group kernel");
    if (q->N <= 0 || q->N > 65535 || q->nnz < 0 || q->n_inst <= 0 || q->npar != sh.np ||
        q->nsteps < 0 || q->nsteps > 0x7fffffff || !(q->dt > 0.0f) || !q->row ||
        (q->nnz > 0 && (!q->col || !q->weights || !q->lengths)) || !q->couplings || !q->speeds ||
        !q->state0 || !q->nparam || (q->flags & ~TVBG_F_NOISE) || q->rounding < 0 || q->rounding > 2)
        return set_error(TVBG_EINVAL, "tvbg_serve_admit: bad request");
    if ((q->flags & TVBG_F_NOISE) && sh.ns > 4)
        return set_error(TVBG_EUNSUPPORTED, "tvbg_serve_admit: noise on more than 4 state variables");
    Request* r = new (std::nothrow) Request;
    if (!r) return set_error(TVBG_EINVAL, "tvbg_serve_admit: out of host memory");
    r->model = q->model;
    r->cfun = q->cfun;
    r->N = q->N;
    r->nnz = q->nnz;
    r->n_inst = q->n_inst;
    r->npar = q->npar;
    r->shape = sh;
    r->nsteps = q->nsteps;
    r->dt = q->dt;
    r->seed = q->seed;
    r->flags = q->flags;
    r->cf_b = q->cf_b;
    std::memcpy(r->cf_p, q->cf_p, sizeof(r->cf_p));
    std::memcpy(r->sigma, q->sigma, sizeof(r->sigma));
    std::memcpy(r->consts, q->consts, sizeof(r->consts));
    r->channels = kuramoto ? 2 : 1;
    r->couplings.assign(q->couplings, q->couplings + q->n_inst);
    r->state0.assign(q->state0, q->state0 + static_cast<size_t>(q->n_inst) * q->N * sh.ns);
    r->nparam.assign(q->nparam, q->nparam + static_cast<size_t>(q->n_inst) * q->N * sh.np);
    int rc = plan(*r, *q);
    if (rc == TVBG_OK && static_cast<int64_t>(r->bytes) > p->cap)
        rc = set_error(TVBG_EINVAL, "tvbg_serve_admit: the request alone exceeds the budget");
    if (rc) {
        delete r;
        return rc;
    }
    r->id = p->next_id++;
    p->queue.push_back(r);
    p->all[r->id] = r;
    *id = r->id;
    return TVBG_OK;
}

// A rolling tick: admit what fits, launch a chunk for every active request
// with none running, wait (at most 20 ms) until some chunk is done when none
// is yet, then take every finished chunk -- status word, clock, retirement
// -- and relaunch its request at once.  Requests advance at their own pace:
// no request waits for the slowest chunk of the others.
int tvbg_serve_tick(tvbg_serve* p, int32_t* n_active, int32_t* n_queued) {
    if (!p) return set_error(TVBG_EINVAL, "tvbg_serve_tick: null");
    if (p->cta_cap < 0) {  // -1: about three waves of CTAs resident at once
        int dev = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve_tick: SM count");
        p->cta_cap = 3 * static_cast<int64_t>(sms);
    }
    // admit in arrival order while the budget, the device and the CTA cap
    // allow (an empty pool always admits its next request)
    while (!p->queue.empty()) {
        Request* r = p->queue.front();
        size_t free_b = 0, total_b = 0;
        cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_serve_tick: cudaMemGetInfo");
        if (p->used + static_cast<int64_t>(r->bytes) > p->budget || r->bytes > free_b) break;
        const int64_t ctas = static_cast<int64_t>(r->members.size()) * r->cluster;
        if (p->cta_cap > 0 && !p->active.empty() && p->active_ctas + ctas > p->cta_cap) break;
        int rc = materialise(*p, *r);
        if (rc) {
            release(*p, *r);
            return rc;
        }
        p->queue.pop_front();
        p->used += static_cast<int64_t>(r->bytes);
        p->active_ctas += r->ctas;
        r->status = TVBG_SERVE_ACTIVE;
        p->active.push_back(r);
    }
    uint64_t mark;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        mark = p->completions;
    }
    int rc = launch_idle(*p);
    if (rc) return rc;
    // finished chunks (a chunk counted after `mark` wakes the wait below;
    // one counted before it is already seen by its event)
    auto finished = [&](Request& r, bool* done) -> int {
        *done = false;
        if (!r.inflight) {
            *done = r.done >= r.nsteps;  // zero steps: retire without a chunk
            return TVBG_OK;
        }
        const cudaError_t q = cudaEventQuery(r.done_ev);
        if (q == cudaErrorNotReady) return TVBG_OK;
        if (q != cudaSuccess) return set_cuda_error(q, "tvbg_serve_tick: event");
        *done = true;
        return TVBG_OK;
    };
    bool any = false;
    for (Request* r : p->active) {
        bool d = false;
        if ((rc = finished(*r, &d))) return rc;
        any = any || d;
    }
    if (!any) {
        bool running = false;
        for (const Request* r : p->active) running = running || r->inflight > 0;
        if (running) {
            std::unique_lock<std::mutex> lk(p->mu);
            p->cv.wait_for(lk, std::chrono::milliseconds(20), [&] { return p->completions != mark; });
        }
    }
    // take the finished chunks: status words first (an error leaves the
    // request as it was), then clocks and retirement; the active list is
    // rebuilt before any return, so a released request never stays in it
    std::vector<Request*> keep;
    for (size_t i = 0; i < p->active.size(); ++i) {
        Request& r = *p->active[i];
        bool d = false;
        if (rc == TVBG_OK) rc = finished(r, &d);
        if (rc == TVBG_OK && d && r.inflight) {
            if (*r.h_status != 0) {
                rc = set_error(TVBG_EDEVICE, "tvbg_serve_tick: a group kernel reported an error");
            } else {
                r.done += r.inflight;
                r.inflight = 0;
            }
        }
        if (rc == TVBG_OK && d && r.done >= r.nsteps) {
            rc = collect(r);
            if (rc == TVBG_OK) {
                release(*p, r);
                p->used -= static_cast<int64_t>(r.bytes);
                p->active_ctas -= r.ctas;
                r.status = TVBG_SERVE_DONE;
                p->finished.push_back(r.id);
                continue;
            }
        }
        keep.push_back(&r);
    }
    p->active.swap(keep);
    if (rc) return rc;
    rc = launch_idle(*p);  // the finished chunks' requests run on at once
    if (rc) return rc;
    if (n_active) *n_active = static_cast<int32_t>(p->active.size());
    if (n_queued) *n_queued = static_cast<int32_t>(p->queue.size());
    return TVBG_OK;
}

int tvbg_serve_finished(tvbg_serve* p, int64_t* ids, int32_t cap, int32_t* n) {
    if (!p || !n || cap < 0 || (cap > 0 && !ids)) return set_error(TVBG_EINVAL, "tvbg_serve_finished: bad arguments");
    const size_t k = std::min<size_t>(static_cast<size_t>(cap), p->finished.size());
    std::copy(p->finished.begin(), p->finished.begin() + k, ids);
    p->finished.erase(p->finished.begin(), p->finished.begin() + k);
    *n = static_cast<int32_t>(k);
    return TVBG_OK;
}

int tvbg_serve_poll(tvbg_serve* p, int64_t id, int32_t* status, float* state_out) {
    if (!p || !status) return set_error(TVBG_EINVAL, "tvbg_serve_poll: null");
    auto it = p->all.find(id);
    if (it == p->all.end()) return set_error(TVBG_EINVAL, "tvbg_serve_poll: unknown id");
    const Request& r = *it->second;
    *status = r.status;
    if (r.status == TVBG_SERVE_DONE && state_out)
        std::memcpy(state_out, r.result.data(), r.result.size() * sizeof(float));
    return TVBG_OK;
}

int tvbg_serve_cancel(tvbg_serve* p, int64_t id) {
    if (!p) return set_error(TVBG_EINVAL, "tvbg_serve_cancel: null");
    auto it = p->all.find(id);
    if (it == p->all.end()) return set_error(TVBG_EINVAL, "tvbg_serve_cancel: unknown id");
    Request* r = it->second;
    if (r->status == TVBG_SERVE_QUEUED) {
        p->queue.erase(std::find(p->queue.begin(), p->queue.end(), r));
    } else if (r->status == TVBG_SERVE_ACTIVE) {
        p->active.erase(std::find(p->active.begin(), p->active.end(), r));
        release(*p, *r);
        p->used -= static_cast<int64_t>(r->bytes);
        p->active_ctas -= r->ctas;
    } else {
        return set_error(TVBG_EINVAL, "tvbg_serve_cancel: the request is done or cancelled");
    }
    r->status = TVBG_SERVE_CANCELLED;
    return TVBG_OK;
}

int tvbg_serve_progress(tvbg_serve* p, int64_t id, int64_t* steps_done) {
    if (!p || !steps_done) return set_error(TVBG_EINVAL, "tvbg_serve_progress: null");
    auto it = p->all.find(id);
    if (it == p->all.end()) return set_error(TVBG_EINVAL, "tvbg_serve_progress: unknown id");
    *steps_done = it->second->done;
    return TVBG_OK;
}

int tvbg_serve_issued(tvbg_serve* p, int64_t id, int64_t* steps) {
    if (!p || !steps) return set_error(TVBG_EINVAL, "tvbg_serve_issued: null");
    auto it = p->all.find(id);
    if (it == p->all.end()) return set_error(TVBG_EINVAL, "tvbg_serve_issued: unknown id");
    *steps = it->second->done + it->second->inflight;
    return TVBG_OK;
}

int tvbg_serve_set_concurrency(tvbg_serve* p, int64_t max_ctas) {
    if (!p) return set_error(TVBG_EINVAL, "tvbg_serve_set_concurrency: null");
    p->cta_cap = max_ctas < 0 ? -1 : max_ctas;
    return TVBG_OK;
}

int tvbg_serve_set_budget(tvbg_serve* p, int64_t budget) {
    if (!p || budget < 0) return set_error(TVBG_EINVAL, "tvbg_serve_set_budget: bad arguments");
    p->budget = budget < p->cap ? budget : p->cap;
    return TVBG_OK;
}

int tvbg_serve_usage(tvbg_serve* p, int64_t id, int64_t* used, int64_t* footprint) {
    if (!p) return set_error(TVBG_EINVAL, "tvbg_serve_usage: null");
    if (used) *used = p->used;
    if (footprint) {
        auto it = p->all.find(id);
        *footprint = it == p->all.end() ? -1 : static_cast<int64_t>(it->second->bytes);
    }
    return TVBG_OK;
}

}  // extern "C"
