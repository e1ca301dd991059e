// batch_attn.cpp -- the batched attention engine (mcAttnBatch*): host C++
// over the library's own C entry points, no PyTorch.
//
// Create: the instances' plain vector CSRs are stacked into one
// block-diagonal mask on the host (rows back to back, every instance's
// columns offset by its first token), converted by the host packer
// (mcAlignRowOffsets, mcPadColumnIndices, mcSortedRowSwizzle) and uploaded
// once, with the buffer of the quantized Q/K/V and a status word.  Run:
// mcQuantize, then mcSparseAttention over every (vector-row, head) item.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>
#include <vector>

#include "../../include/magicube_gb300.h"
#include "mc_host.h"

struct mcAttnBatch {
    int n_instances = 0, V = 8, heads = 0, d = 64, lb = 8, rb = 8, requant = MC_REQUANT_FIXED;
    float scale_qkv = 1.f, scale_sfmx = 1.f;
    int m_vec = 0, max_row_nnz = 0;
    long long tokens = 0;
    std::vector<long long> token_offsets;
    int* row_indices = nullptr;
    int* pairs = nullptr;
    int* cols = nullptr;
    void* qkv_q = nullptr;        // [3][heads][tokens * d * rb / 8] bytes
    int* status = nullptr;
    int warps = 0, stages = 0, ctas_per_sm = 0;  // fused launch configuration (0 = default)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void release(mcAttnBatch* b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->row_indices);
    cudaFree(b->pairs);
    cudaFree(b->cols);
    cudaFree(b->qkv_q);
    cudaFree(b->status);
    delete b;
}

int upload(int** dst, const std::vector<int>& src)
{
    const size_t n = std::max<size_t>(src.size(), 1);
    int rc = (int)cudaMalloc(reinterpret_cast<void**>(dst), n * sizeof(int));
    if (rc) return rc;
    if (src.empty()) return (int)cudaMemset(*dst, 0xff, sizeof(int));  // one -1 column: nothing stored
    return (int)cudaMemcpy(*dst, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice);
}

int check_desc(const mcAttnBatchDesc& d)
{
    if (d.n_instances < 1 || !d.seq_lens || !d.row_offsets || !d.col_indices)
        return mc::fail(1, "mcAttnBatchCreate: need at least one instance with lengths, offsets and columns");
    if (!(d.vec_length == 2 || d.vec_length == 4 || d.vec_length == 8))
        return mc::fail(1, "mcAttnBatchCreate: vec_length must be 2, 4 or 8");
    if (d.head_dim != 64 || d.heads < 1) return mc::fail(1, "mcAttnBatchCreate: head_dim must be 64, heads >= 1");
    if (!((d.lhs_bits == 8 && d.rhs_bits == 8) || (d.lhs_bits == 16 && d.rhs_bits == 8) ||
          (d.lhs_bits == 8 && d.rhs_bits == 4)))
        return mc::fail(1, "mcAttnBatchCreate: pairs L8-R8, L16-R8 and L8-R4");
    if (d.requant != MC_REQUANT_FIXED && d.requant != MC_REQUANT_ROWMAX)
        return mc::fail(1, "mcAttnBatchCreate: invalid requant mode");
    if (d.requant == MC_REQUANT_ROWMAX && d.lhs_bits != 8)
        return mc::fail(1, "mcAttnBatchCreate: row-max requantization writes 8-bit probabilities");
    if (!(d.scale_qkv > 0.f) || !(d.scale_sfmx > 0.f))
        return mc::fail(1, "mcAttnBatchCreate: scales must be positive");
    return 0;
}

// The instances' CSRs stacked into one block-diagonal plain CSR (host):
// ro (m + 1 offsets), ci (columns offset by each instance's first token),
// toks (token offsets, n_instances + 1).
int stack_masks(const mcAttnBatchDesc& d, std::vector<int>& ro, std::vector<int>& ci, std::vector<long long>& toks)
{
    const int V = d.vec_length;
    ro.assign(1, 0);
    ci.clear();
    toks.assign(1, 0);
    for (int i = 0; i < d.n_instances; ++i) {
        const int L = d.seq_lens[i];
        if (L <= 0 || L % V) return mc::fail(1, "mcAttnBatchCreate: every length must be a positive multiple of V");
        if (!d.row_offsets[i] || !d.col_indices[i]) return mc::fail(1, "mcAttnBatchCreate: null instance mask");
        const int mv = L / V;
        const int* r = d.row_offsets[i];
        if (r[0] != 0) return mc::fail(1, "mcAttnBatchCreate: an instance's offsets must start at 0");
        const long long base = ro.back(), tok = toks.back();
        for (int v = 0; v < mv; ++v) {
            if (r[v + 1] < r[v]) return mc::fail(1, "mcAttnBatchCreate: offsets must not decrease");
            for (int j = r[v]; j < r[v + 1]; ++j) {
                const int c = d.col_indices[i][j];
                if (c < 0 || c >= L) return mc::fail(1, "mcAttnBatchCreate: a column lies outside its instance");
                ci.push_back((int)(c + tok));
            }
            if (base + r[v + 1] > 0x7fffffffLL) return mc::fail(1, "mcAttnBatchCreate: too many nonzero vectors");
            ro.push_back((int)(base + r[v + 1]));
        }
        toks.push_back(tok + L);
    }
    if (toks.back() > 0x7fffffffLL) return mc::fail(1, "mcAttnBatchCreate: too many tokens");
    return 0;
}

mcAttnBatch* new_batch(const mcAttnBatchDesc& d, int m, int longest, const std::vector<long long>& toks)
{
    mcAttnBatch* b = new (std::nothrow) mcAttnBatch;
    if (!b) return nullptr;
    b->n_instances = d.n_instances;
    b->V = d.vec_length;
    b->heads = d.heads;
    b->d = d.head_dim;
    b->lb = d.lhs_bits;
    b->rb = d.rhs_bits;
    b->requant = d.requant;
    b->scale_qkv = d.scale_qkv;
    b->scale_sfmx = d.scale_sfmx;
    b->m_vec = m;
    b->max_row_nnz = longest;
    b->tokens = toks.back();
    b->token_offsets = toks;
    return b;
}

int longest_row(const std::vector<int>& ro)
{
    int longest = 0;
    for (size_t v = 0; v + 1 < ro.size(); ++v) longest = std::max(longest, ro[v + 1] - ro[v]);
    return longest;
}

}  // namespace

extern "C" {

int mcAttnBatchCreate(const mcAttnBatchDesc* desc, mcAttnBatch** batch)
{
    mc::clear_error();
    if (!desc || !batch) return mc::fail(1, "mcAttnBatchCreate: null argument");
    *batch = nullptr;
    const mcAttnBatchDesc& d = *desc;
    if (int rc = check_desc(d)) return rc;
    std::vector<int> ro, ci;
    std::vector<long long> toks;
    if (int rc = stack_masks(d, ro, ci, toks)) return rc;
    const int m = (int)(ro.size() - 1);
    const int align = d.rhs_bits == 8 ? 16 : 32;
    std::vector<int> pairs(2 * (size_t)m), ri(std::max(m, 1));
    const int n_al = mcAlignRowOffsets(m, ro.data(), align, pairs.data());
    if (n_al < 0) return mc::fail(1, "mcAttnBatchCreate: aligned slot count overflows");
    std::vector<int> cols(std::max<size_t>((size_t)n_al, 1), -1);
    if (int rc = mcPadColumnIndices(m, ro.data(), ci.empty() ? nullptr : ci.data(), pairs.data(), n_al, 0,
                                    cols.data()))
        return rc;
    if (int rc = mcSortedRowSwizzle(m, ro.data(), ri.data())) return rc;
    const int longest = longest_row(ro);
    if (longest > 4096) return mc::fail(1, "mcAttnBatchCreate: rows of at most 4096 nonzero vectors");

    mcAttnBatch* b = new_batch(d, m, longest, toks);
    if (!b) return mc::fail(1, "mcAttnBatchCreate: out of host memory");
    int rc = upload(&b->row_indices, ri);
    if (!rc) rc = upload(&b->pairs, pairs);
    if (!rc) rc = upload(&b->cols, std::vector<int>(cols.begin(), cols.begin() + n_al));
    if (!rc)
        rc = (int)cudaMalloc(&b->qkv_q,
                             std::max<size_t>((size_t)3 * d.heads * b->tokens * d.head_dim * d.rhs_bits / 8, 16));
    if (!rc) rc = (int)cudaMalloc(reinterpret_cast<void**>(&b->status), sizeof(int));
    if (!rc) rc = (int)cudaMemset(b->status, 0, sizeof(int));
    if (rc) {
        release(b);
        return rc;
    }
    *batch = b;
    return 0;
}

int mcAttnBatchTokens(const mcAttnBatch* b, long long* token_offsets)
{
    mc::clear_error();
    if (!b || !token_offsets) return mc::fail(1, "mcAttnBatchTokens: null argument");
    std::copy(b->token_offsets.begin(), b->token_offsets.end(), token_offsets);
    return 0;
}

namespace {

int run(mcAttnBatch* b, const void* qkv, void* out, cudaStream_t s, int warps, int stages, int ctas)
{
    const long long per_head = b->tokens * b->d;
    if (int rc = mcQuantize(qkv, b->qkv_q, 3 * b->heads * per_head, b->rb, b->scale_qkv, s)) return rc;
    const long long head_bytes = per_head * b->rb / 8;
    const uint8_t* q = static_cast<const uint8_t*>(b->qkv_q);
    const bool rowmax = b->requant == MC_REQUANT_ROWMAX;
    mcAttnDesc a{};
    a.m_vec = b->m_vec;
    a.vec_length = b->V;
    a.heads = b->heads;
    a.head_dim = b->d;
    a.max_row_nnz = b->max_row_nnz;
    a.lhs_bits = b->lb;
    a.rhs_bits = b->rb;
    a.requant = b->requant;
    a.score_scale = b->scale_qkv * b->scale_qkv;
    a.scaling = 1.0f / std::sqrt((float)b->d);
    a.prob_scale = b->scale_sfmx;
    a.out_scale = rowmax ? b->scale_qkv : b->scale_qkv * b->scale_sfmx;
    a.row_indices = b->row_indices;
    a.row_offsets = b->pairs;
    a.column_indices = b->cols;
    a.q = q;
    a.k = q + b->heads * head_bytes;
    a.v = q + 2 * b->heads * head_bytes;
    a.head_stride = head_bytes;
    a.out = out;
    a.out_head_stride = per_head;
    a.status = b->status;
    a.warps = warps;
    a.stages = stages;
    a.ctas_per_sm = ctas;
    return mcSparseAttention(&a, s);
}

}  // namespace

int mcAttnBatchRun(mcAttnBatch* b, const void* qkv, void* out, cudaStream_t stream)
{
    mc::clear_error();
    if (!b || !qkv || !out) return mc::fail(1, "mcAttnBatchRun: null argument");
    return run(b, qkv, out, stream, b->warps, b->stages, b->ctas_per_sm);
}

int mcAttnBatchTune(mcAttnBatch* b, const void* qkv, void* out, cudaStream_t stream, int* warps, int* stages,
                    int* ctas_per_sm)
{
    mc::clear_error();
    if (!b || !qkv || !out) return mc::fail(1, "mcAttnBatchTune: null argument");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = (int)cudaEventCreate(&e0);
    if (!rc) rc = (int)cudaEventCreate(&e1);
    float best = 0.f;
    int bw = 0, bs = 0, bc = 0;
    bool found = false;
    for (int w : {4, 8})
        for (int st : {2, 3})
            for (int c : {0, 2, 4}) {
                if (rc) break;
                if (run(b, qkv, out, stream, w, st, c)) {  // a configuration that does not apply
                    cudaGetLastError();
                    continue;
                }
                rc = (int)cudaEventRecord(e0, stream);
                for (int r = 0; r < 5 && !rc; ++r) rc = run(b, qkv, out, stream, w, st, c);
                if (!rc) rc = (int)cudaEventRecord(e1, stream);
                if (!rc) rc = (int)cudaEventSynchronize(e1);
                float ms = 0.f;
                if (!rc) rc = (int)cudaEventElapsedTime(&ms, e0, e1);
                if (!rc && (!found || ms < best)) {
                    best = ms;
                    bw = w;
                    bs = st;
                    bc = c;
                    found = true;
                }
            }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return rc;
    if (!found) return mc::fail(1, "mcAttnBatchTune: no launch configuration applies");
    b->warps = bw;
    b->stages = bs;
    b->ctas_per_sm = bc;
    if (warps) *warps = bw;
    if (stages) *stages = bs;
    if (ctas_per_sm) *ctas_per_sm = bc;
    return 0;
}

int mcAttnBatchCapture(mcAttnBatch* b, const void* qkv, void* out, cudaStream_t stream)
{
    mc::clear_error();
    if (!b || !qkv || !out) return mc::fail(1, "mcAttnBatchCapture: null argument");
    if (!stream) return mc::fail(1, "mcAttnBatchCapture: capture needs a created stream, not the legacy default stream");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    int rc = (int)cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (rc) return rc;
    const int rr = run(b, qkv, out, stream, b->warps, b->stages, b->ctas_per_sm);
    cudaGraph_t g = nullptr;
    rc = (int)cudaStreamEndCapture(stream, &g);
    if (rr) {
        if (g) cudaGraphDestroy(g);
        return rr;
    }
    if (rc) return rc;
    b->graph = g;
    return (int)cudaGraphInstantiate(&b->exec, g, 0);
}

int mcAttnBatchReplay(mcAttnBatch* b, cudaStream_t stream)
{
    mc::clear_error();
    if (!b || !b->exec) return mc::fail(1, "mcAttnBatchReplay: nothing captured");
    return (int)cudaGraphLaunch(b->exec, stream);
}

int mcAttnBatchStatus(mcAttnBatch* b, int* status)
{
    mc::clear_error();
    if (!b || !status) return mc::fail(1, "mcAttnBatchStatus: null argument");
    return (int)cudaMemcpy(status, b->status, sizeof(int), cudaMemcpyDeviceToHost);
}

void mcAttnBatchDestroy(mcAttnBatch* b) { release(b); }

}  // extern "C"
