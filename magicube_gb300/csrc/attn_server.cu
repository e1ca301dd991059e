// attn_server.cu -- the attention request server (mcAttnServer*): a host C++
// continuous-batching loop over the library's own device entry points.
//
// Requests arrive on the host clock; waiting requests are admitted in arrival
// order as one batch per free slot (a non-blocking stream), when the batch's
// device memory fits the admission budget (free memory plus what the
// stream-ordered pool holds unused, less the reserve and less the batches
// already in flight).  A batch is assembled
// entirely on its stream:
//   1. one stream-ordered allocation for every buffer of the batch;
//   2. stack_masks_kernel: the requests' plain CSRs into one block-diagonal
//      CSR (row offsets shifted by the nonzeros before, columns by the tokens
//      before, columns clamped into their own sequence);
//   3. mcDevicePack: aligned pairs, padded columns, longest-first row order;
//   4. Q/K/V staged into [3][heads][T][64] with one 2-D copy per request,
//      mcQuantize, mcSparseAttention (the fused kernel), outputs copied back
//      into each request's buffer with one 2-D copy each;
//   5. the allocation freed on the stream, an event recorded.
// Completions are polled with cudaEventQuery, so batches on different slots
// overlap on the device while the host admits the next.
#include <cuda_fp16.h>
#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <new>
#include <thread>
#include <vector>

#include "../../include/magicube_gb300.h"
#include "mc_host.h"

struct mcAttnServer {
    mcAttnServerDesc d{};
    std::vector<cudaStream_t> streams;
    int* status_host = nullptr;  // pinned: one fused-kernel status word per slot
};

namespace {

struct StackReq {
    const int* ro;
    const int* ci;
    int m, nnz, seq_len;
    int row_off, nnz_off, tok_off;
};

// Block-diagonal stacking of the batch's requests (blockIdx.y = request):
// offsets shifted by the nonzeros of the earlier requests (and clamped into
// the request's own nonzeros), columns shifted by the earlier tokens (and
// clamped into the request's own sequence), so that inconsistent input
// cannot send the packer or the attention kernel outside the batch.
__global__ void stack_masks_kernel(const StackReq* __restrict__ reqs, int* __restrict__ ro_out,
                                   int* __restrict__ ci_out)
{
    const StackReq q = reqs[blockIdx.y];
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < q.m; v += stride) {
        const int o = __ldg(q.ro + v + 1);
        ro_out[q.row_off + v + 1] = q.nnz_off + (o < 0 ? 0 : (o > q.nnz ? q.nnz : o));
    }
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < q.nnz; j += stride) {
        const int c = __ldg(q.ci + j);
        ci_out[q.nnz_off + j] = q.tok_off + (c < 0 ? 0 : (c >= q.seq_len ? q.seq_len - 1 : c));
    }
    if (blockIdx.y == 0 && blockIdx.x == 0 && threadIdx.x == 0) ro_out[0] = 0;
}

size_t up256(size_t b) { return (b + 255) / 256 * 256; }

// Device memory of one batch: the layout of its single allocation.
struct BatchLayout {
    size_t reqs, ro, ci, pairs, n_al, cols, ri, status, stage, out, qkv_q, total;
    long long cols_cap;
};

BatchLayout layout(const mcAttnServerDesc& d, int n_req, long long tokens, long long rows, long long nnz)
{
    const int align = d.rhs_bits == 8 ? 16 : 32;
    BatchLayout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += up256(bytes);
        return at;
    };
    L.cols_cap = nnz + rows * (align - 1) + 1;
    L.reqs = take(sizeof(StackReq) * (size_t)n_req);
    L.ro = take(4 * (size_t)(rows + 1));
    L.ci = take(4 * (size_t)std::max<long long>(nnz, 1));
    L.pairs = take(8 * (size_t)rows);
    L.n_al = take(4);
    L.cols = take(4 * (size_t)L.cols_cap);
    L.ri = take(4 * (size_t)rows);
    L.status = take(4);
    const size_t plane = (size_t)tokens * d.head_dim;  // elements of one [T][d] plane
    L.stage = take(2 * plane * 3 * d.heads);
    L.out = take(2 * plane * d.heads);
    L.qkv_q = take(plane * 3 * d.heads * d.rhs_bits / 8);
    L.total = o;
    return L;
}

// Device bytes a batch needs: its own allocation plus the packer's scratch
// (tile sums and the radix sort of the row lengths), with a margin for the
// stream-ordered allocator's granularity.
size_t footprint(const BatchLayout& L, long long rows)
{
    const size_t pack = 64 * (size_t)rows + (4u << 20);
    return (size_t)((double)(L.total + pack) * 1.25) + (2u << 20);
}

// The admission budget: free device memory, plus memory the default
// stream-ordered pool holds but no allocation uses (batches that finished
// return theirs there, not to the device, until a synchronisation), less the
// reserve.
int admission_budget(const mcAttnServerDesc& d, long long* avail)
{
    size_t fr = 0, tot = 0;
    if (int rc = (int)cudaMemGetInfo(&fr, &tot)) return rc;
    long long pool_free = 0;
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long reserved = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            pool_free = (long long)(reserved - used);
    }
    cudaGetLastError();  // a missing pool only loses the pool term
    *avail = (long long)fr + pool_free - d.hbm_reserve_bytes;
    return 0;
}

struct Inflight {
    int slot = -1;
    char* mem = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<int> reqs;
    long long bytes = 0;  // the footprint admission charged
};

int check_server_desc(const mcAttnServerDesc& d)
{
    if (!(d.vec_length == 2 || d.vec_length == 4 || d.vec_length == 8))
        return mc::fail(1, "mcAttnServerCreate: vec_length must be 2, 4 or 8");
    if (d.head_dim != 64 || d.heads < 1) return mc::fail(1, "mcAttnServerCreate: head_dim must be 64, heads >= 1");
    if (!((d.lhs_bits == 8 && d.rhs_bits == 8) || (d.lhs_bits == 16 && d.rhs_bits == 8) ||
          (d.lhs_bits == 8 && d.rhs_bits == 4)))
        return mc::fail(1, "mcAttnServerCreate: pairs L8-R8, L16-R8 and L8-R4");
    if (d.requant != MC_REQUANT_FIXED && d.requant != MC_REQUANT_ROWMAX)
        return mc::fail(1, "mcAttnServerCreate: invalid requant mode");
    if (d.requant == MC_REQUANT_ROWMAX && d.lhs_bits != 8)
        return mc::fail(1, "mcAttnServerCreate: row-max requantization writes 8-bit probabilities");
    if (!(d.scale_qkv > 0.f) || !(d.scale_sfmx > 0.f)) return mc::fail(1, "mcAttnServerCreate: scales must be positive");
    if (d.max_batch_tokens < 1) return mc::fail(1, "mcAttnServerCreate: max_batch_tokens must be positive");
    if (d.max_inflight < 1 || d.max_inflight > 8) return mc::fail(1, "mcAttnServerCreate: max_inflight must be 1 .. 8");
    if (d.hbm_reserve_bytes < 0) return mc::fail(1, "mcAttnServerCreate: negative reserve");
    return 0;
}

int check_request(const mcAttnServerDesc& d, const mcAttnRequest& r)
{
    if (r.seq_len <= 0 || r.seq_len % d.vec_length)
        return mc::fail(1, "mcAttnServerRun: every seq_len must be a positive multiple of vec_length");
    if (r.nnz_vec < 0 || r.max_row_nnz < 0 || r.max_row_nnz > 4096)
        return mc::fail(1, "mcAttnServerRun: nnz_vec >= 0 and max_row_nnz in [0, 4096]");
    if (!r.row_offsets || (r.nnz_vec > 0 && !r.col_indices) || !r.qkv || !r.out)
        return mc::fail(1, "mcAttnServerRun: null request pointer");
    if (!(r.arrival_s >= 0.0)) return mc::fail(1, "mcAttnServerRun: arrival times must be >= 0");
    // the stacked CSR and the packer's aligned count are int: one request's
    // nonzeros with its rows' alignment padding must fit
    const long long align = d.rhs_bits == 8 ? 16 : 32;
    if (r.nnz_vec + (long long)(r.seq_len / d.vec_length) * align > INT_MAX)
        return mc::fail(1, "mcAttnServerRun: a request's aligned nonzero count exceeds the int range");
    return 0;
}

// Launches one batch of requests `ids` on `stream` into the allocation `mem`.
int launch_batch(const mcAttnServerDesc& d, const mcAttnRequest* reqs, const std::vector<int>& ids, char* mem,
                 const BatchLayout& L, long long tokens, long long rows, int max_row, cudaStream_t s, int* status_host)
{
    const int V = d.vec_length;
    std::vector<StackReq> sr(ids.size());
    long long row_off = 0, nnz_off = 0, tok_off = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
        const mcAttnRequest& r = reqs[ids[i]];
        sr[i] = StackReq{r.row_offsets, r.col_indices, r.seq_len / V, r.nnz_vec, r.seq_len,
                         (int)row_off, (int)nnz_off, (int)tok_off};
        row_off += r.seq_len / V;
        nnz_off += r.nnz_vec;
        tok_off += r.seq_len;
    }
    StackReq* sr_d = reinterpret_cast<StackReq*>(mem + L.reqs);
    int* ro = reinterpret_cast<int*>(mem + L.ro);
    int* ci = reinterpret_cast<int*>(mem + L.ci);
    int rc = (int)cudaMemcpyAsync(sr_d, sr.data(), sizeof(StackReq) * sr.size(), cudaMemcpyHostToDevice, s);
    if (rc) return rc;
    // the copy above reads pageable host memory: it has been taken by the time the call returns
    long long longest = 1;
    for (const StackReq& q : sr) longest = std::max<long long>(longest, std::max(q.m, q.nnz));
    const unsigned gx = (unsigned)std::min<long long>((longest + 255) / 256, 64);
    stack_masks_kernel<<<dim3(gx, (unsigned)sr.size()), 256, 0, s>>>(sr_d, ro, ci);
    if ((rc = (int)cudaGetLastError())) return rc;

    mcDevicePackDesc pk{};
    pk.m_vec = (int)rows;
    pk.vec_length = V;
    pk.lhs_bits = 0;  // the mask only
    pk.rhs_bits = d.rhs_bits;
    pk.alignment = d.rhs_bits == 8 ? 16 : 32;
    pk.shuffle8 = 0;
    pk.value_layout = MC_VALUES_PACKED;
    pk.sort_rows = 1;
    pk.row_offsets = ro;
    pk.col_indices = ci;
    pk.aligned_pairs = reinterpret_cast<int*>(mem + L.pairs);
    pk.aligned_nnz = reinterpret_cast<int*>(mem + L.n_al);
    pk.out_cols = reinterpret_cast<int*>(mem + L.cols);
    pk.cols_capacity = L.cols_cap;
    pk.row_indices = reinterpret_cast<int*>(mem + L.ri);
    int* status = reinterpret_cast<int*>(mem + L.status);
    if ((rc = (int)cudaMemsetAsync(status, 0, sizeof(int), s))) return rc;
    pk.status = status;
    if ((rc = mcDevicePack(&pk, s))) return rc;

    const size_t plane = (size_t)tokens * d.head_dim;
    __half* stage = reinterpret_cast<__half*>(mem + L.stage);
    __half* out = reinterpret_cast<__half*>(mem + L.out);
    tok_off = 0;
    for (int id : ids) {
        const mcAttnRequest& r = reqs[id];
        const size_t row_bytes = (size_t)r.seq_len * d.head_dim * 2;
        rc = (int)cudaMemcpy2DAsync(stage + (size_t)tok_off * d.head_dim, plane * 2, r.qkv, row_bytes, row_bytes,
                                    (size_t)3 * d.heads, cudaMemcpyDeviceToDevice, s);
        if (rc) return rc;
        tok_off += r.seq_len;
    }
    uint8_t* q = reinterpret_cast<uint8_t*>(mem + L.qkv_q);
    if ((rc = mcQuantize(stage, q, (long long)(3 * d.heads * plane), d.rhs_bits, d.scale_qkv, s))) return rc;
    const long long head_bytes = (long long)plane * d.rhs_bits / 8;
    const bool rowmax = d.requant == MC_REQUANT_ROWMAX;
    mcAttnDesc a{};
    a.m_vec = (int)rows;
    a.vec_length = V;
    a.heads = d.heads;
    a.head_dim = d.head_dim;
    a.max_row_nnz = std::max(max_row, 1);
    a.lhs_bits = d.lhs_bits;
    a.rhs_bits = d.rhs_bits;
    a.requant = d.requant;
    a.score_scale = d.scale_qkv * d.scale_qkv;
    a.scaling = 1.0f / std::sqrt((float)d.head_dim);
    a.prob_scale = d.scale_sfmx;
    a.out_scale = rowmax ? d.scale_qkv : d.scale_qkv * d.scale_sfmx;
    a.row_indices = pk.row_indices;
    a.row_offsets = pk.aligned_pairs;
    a.column_indices = pk.out_cols;
    a.q = q;
    a.k = q + d.heads * head_bytes;
    a.v = q + 2 * d.heads * head_bytes;
    a.head_stride = head_bytes;
    a.out = out;
    a.out_head_stride = (long long)plane;
    a.status = status;
    if ((rc = mcSparseAttention(&a, s))) return rc;
    tok_off = 0;
    for (int id : ids) {
        const mcAttnRequest& r = reqs[id];
        const size_t row_bytes = (size_t)r.seq_len * d.head_dim * 2;
        rc = (int)cudaMemcpy2DAsync(r.out, row_bytes, out + (size_t)tok_off * d.head_dim, plane * 2, row_bytes,
                                    (size_t)d.heads, cudaMemcpyDeviceToDevice, s);
        if (rc) return rc;
        tok_off += r.seq_len;
    }
    return (int)cudaMemcpyAsync(status_host, status, sizeof(int), cudaMemcpyDeviceToHost, s);
}

}  // namespace

extern "C" {

int mcAttnServerCreate(const mcAttnServerDesc* desc, mcAttnServer** server)
{
    mc::clear_error();
    if (!desc || !server) return mc::fail(1, "mcAttnServerCreate: null argument");
    *server = nullptr;
    if (int rc = check_server_desc(*desc)) return rc;
    mcAttnServer* sv = new (std::nothrow) mcAttnServer;
    if (!sv) return mc::fail(1, "mcAttnServerCreate: out of host memory");
    sv->d = *desc;
    int rc = (int)cudaMallocHost(reinterpret_cast<void**>(&sv->status_host), sizeof(int) * 8);
    for (int i = 0; i < desc->max_inflight && !rc; ++i) {
        cudaStream_t s = nullptr;
        rc = (int)cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (!rc) sv->streams.push_back(s);
    }
    if (rc) {
        mcAttnServerDestroy(sv);
        return rc;
    }
    *server = sv;
    return 0;
}

int mcAttnServerRun(mcAttnServer* sv, const mcAttnRequest* reqs, int n, double* latency_ms, mcAttnServeStats* stats)
{
    using clock = std::chrono::steady_clock;
    mc::clear_error();
    if (!sv || n < 0 || (n > 0 && (!reqs || !latency_ms))) return mc::fail(1, "mcAttnServerRun: invalid arguments");
    const mcAttnServerDesc& d = sv->d;
    for (int i = 0; i < n; ++i)
        if (int rc = check_request(d, reqs[i])) return rc;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [reqs](int a, int b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
    for (int i = 0; i < n; ++i) latency_ms[i] = -1.0;

    mcAttnServeStats st{};
    std::vector<Inflight> inflight;
    std::vector<char> slot_busy(sv->streams.size(), 0);
    std::vector<int> queue;  // arrived, not yet admitted (arrival order)
    size_t next = 0;         // next request of `order` to arrive
    int finished = 0;
    bool held = false;
    int rc = 0, kernel_status = 0;
    const auto t0 = clock::now();
    auto now_s = [&]() { return std::chrono::duration<double>(clock::now() - t0).count(); };

    while (finished < n && !rc) {
        bool progress = false;
        const double now = now_s();
        while (next < (size_t)n && reqs[order[next]].arrival_s <= now) queue.push_back(order[next++]);
        // completions
        for (size_t i = 0; i < inflight.size();) {
            const cudaError_t q = cudaEventQuery(inflight[i].done);
            if (q == cudaErrorNotReady) {
                ++i;
                continue;
            }
            if (q != cudaSuccess) {
                rc = (int)q;
                break;
            }
            const double t = now_s();
            for (int r : inflight[i].reqs) latency_ms[r] = (t - reqs[r].arrival_s) * 1e3;
            finished += (int)inflight[i].reqs.size();
            st.served += (int)inflight[i].reqs.size();
            kernel_status |= sv->status_host[inflight[i].slot];
            cudaEventDestroy(inflight[i].done);
            slot_busy[inflight[i].slot] = 0;
            inflight.erase(inflight.begin() + (long)i);
            progress = true;
        }
        if (rc) break;
        // admissions
        while (!queue.empty() && inflight.size() < sv->streams.size()) {
            std::vector<int> ids;
            long long tokens = 0, rows = 0, nnz = 0;
            int max_row = 0;
            for (int r : queue) {
                const mcAttnRequest& q = reqs[r];
                if (!ids.empty() && tokens + q.seq_len > d.max_batch_tokens) break;
                const long long align = d.rhs_bits == 8 ? 16 : 32;
                if (!ids.empty() && nnz + q.nnz_vec + (rows + q.seq_len / d.vec_length) * align > INT_MAX) break;
                ids.push_back(r);
                tokens += q.seq_len;
                rows += q.seq_len / d.vec_length;
                nnz += q.nnz_vec;
                max_row = std::max(max_row, q.max_row_nnz);
            }
            // Batches already in flight are charged at their full footprint: their
            // stream-ordered allocations need not show in the device's figures yet
            // (conservative when they do; exact with nothing in flight).
            long long avail = 0;
            if ((rc = admission_budget(d, &avail))) break;
            for (const Inflight& f : inflight) avail -= f.bytes;
            BatchLayout L = layout(d, (int)ids.size(), tokens, rows, nnz);
            // shrink the batch from the back until it fits (or one request is left)
            while ((long long)footprint(L, rows) > avail && ids.size() > 1) {
                const mcAttnRequest& q = reqs[ids.back()];
                ids.pop_back();
                tokens -= q.seq_len;
                rows -= q.seq_len / d.vec_length;
                nnz -= q.nnz_vec;
                max_row = 0;
                for (int r : ids) max_row = std::max(max_row, reqs[r].max_row_nnz);
                L = layout(d, (int)ids.size(), tokens, rows, nnz);
            }
            if ((long long)footprint(L, rows) > avail) {
                if (inflight.empty()) {  // does not fit even alone on an idle device: rejected, never launched
                    latency_ms[ids[0]] = -1.0;
                    ++st.rejected;
                    ++finished;
                    queue.erase(queue.begin());
                    progress = true;
                    continue;
                }
                if (!held) ++st.held_back;  // wait for a batch to finish and free its memory
                held = true;
                break;
            }
            held = false;
            int slot = 0;
            while (slot_busy[slot]) ++slot;
            cudaStream_t s = sv->streams[slot];
            Inflight f;
            f.slot = slot;
            f.reqs = ids;
            f.bytes = (long long)footprint(L, rows);
            if ((rc = (int)cudaMallocAsync(reinterpret_cast<void**>(&f.mem), L.total, s))) break;
            rc = launch_batch(d, reqs, ids, f.mem, L, tokens, rows, max_row, s, sv->status_host + slot);
            const int rf = (int)cudaFreeAsync(f.mem, s);
            if (!rc) rc = rf;
            if (!rc) rc = (int)cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
            if (!rc) rc = (int)cudaEventRecord(f.done, s);
            if (rc) {
                // what this batch queued is not tracked: let it drain before returning
                cudaStreamSynchronize(s);
                if (f.done) cudaEventDestroy(f.done);
                break;
            }
            slot_busy[slot] = 1;
            inflight.push_back(f);
            queue.erase(queue.begin(), queue.begin() + (long)ids.size());
            ++st.batches;
            st.max_inflight_seen = std::max(st.max_inflight_seen, (int)inflight.size());
            progress = true;
        }
        if (rc || progress) continue;
        // idle: sleep until the next arrival, or poll the batches on the device
        if (inflight.empty() && queue.empty() && next < (size_t)n) {
            const double wait = reqs[order[next]].arrival_s - now_s();
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
    // on an error, wait for what is still on the device before returning
    for (Inflight& f : inflight) {
        cudaEventSynchronize(f.done);
        cudaEventDestroy(f.done);
    }
    if (rc) return rc;
    st.makespan_s = now_s();
    std::vector<double> lat;
    for (int i = 0; i < n; ++i)
        if (latency_ms[i] >= 0) lat.push_back(latency_ms[i]);
    std::sort(lat.begin(), lat.end());
    if (!lat.empty()) {
        auto pct = [&](double p) {
            const double x = p * (double)(lat.size() - 1);
            const size_t i = (size_t)x;
            const double f = x - (double)i;
            return i + 1 < lat.size() ? lat[i] * (1 - f) + lat[i + 1] * f : lat[i];
        };
        st.p50_ms = pct(0.5);
        st.p99_ms = pct(0.99);
        double sum = 0;
        for (double v : lat) sum += v;
        st.mean_ms = sum / (double)lat.size();
    }
    st.req_per_s = st.makespan_s > 0 ? st.served / st.makespan_s : 0.0;
    if (stats) *stats = st;
    if (kernel_status)
        return mc::fail(1, "mcAttnServerRun: a request's max_row_nnz was below its longest vector-row; "
                           "those rows were left unwritten");
    return 0;
}

int mcAttnServerMemory(const mcAttnServer* sv, const mcAttnRequest* reqs, int n, long long* batch_bytes,
                       long long* available_bytes)
{
    mc::clear_error();
    if (!sv || n < 0 || (n > 0 && !reqs)) return mc::fail(1, "mcAttnServerMemory: invalid arguments");
    long long tokens = 0, rows = 0, nnz = 0;
    for (int i = 0; i < n; ++i) {
        if (int rc = check_request(sv->d, reqs[i])) return rc;
        tokens += reqs[i].seq_len;
        rows += reqs[i].seq_len / sv->d.vec_length;
        nnz += reqs[i].nnz_vec;
    }
    if (batch_bytes) *batch_bytes = (long long)footprint(layout(sv->d, std::max(n, 1), tokens, rows, nnz), rows);
    if (available_bytes) return admission_budget(sv->d, available_bytes);
    return 0;
}

void mcAttnServerDestroy(mcAttnServer* sv)
{
    if (!sv) return;
    for (cudaStream_t s : sv->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    if (sv->status_host) cudaFreeHost(sv->status_host);
    delete sv;
}

}  // extern "C"
