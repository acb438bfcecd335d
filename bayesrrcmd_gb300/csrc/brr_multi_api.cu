// C ABI of the uneven batch: independent regressions of different sizes
// (each its own genotypes, phenotype, seed, marker kind) swept together by one
// cooperative launch of k_sweep_multi per iteration, each instance on its own
// group of CTAs.  Per instance the iteration is the single-chain one
// (BayesRBase::runGibbs loop body, src/BayesRBase.cpp:186-247) through the
// phases of brr_ctx.h.
//
// The autotuner chooses, per instance, the round width (markers resolved per
// grid round) and the number of CTAs: it runs real iterations, reads each
// instance's sweep time from the device timer, keeps the fastest round width
// and then moves CTAs to the instances that finish last until the times are
// balanced (an instance's slices must fit shared memory, which bounds its
// CTAs from below).  Slicing and round width change only the order of
// floating-point sums, never the chain's draws.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "brr_ctx.h"
#include "brr_device.cuh"
#include "brr_internal.h"

using namespace brr;

namespace {

#define MULTI_CUDA(call)                                                                                \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return api_fail(BRR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

constexpr int kChunkInd = 64;   // individuals per slice chunk (16 bytes of codes)

}  // namespace

struct brr_multi {
    int n = 0, form = 0, dev = 0, sms = 0, kmax = 2;
    size_t smem_limit = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    cudaEvent_t done = nullptr;
    std::vector<cudaEvent_t> ready;
    std::vector<brr_ctx *> inst;
    unsigned long long *d_t = nullptr;       // [n][2] device timer at sweep start and end
    unsigned long long *h_t = nullptr;       // pinned copy
    cudaGraphExec_t exec = nullptr;          // the iteration's graph, updated each iteration
    std::vector<double> inst_ms;             // last sweep time of each instance
    double last_sweep_ms = 0.0, last_total_ms = 0.0;
    bool inited = false;
};

namespace {

void free_multi(brr_multi *m)
{
    for (brr_ctx *c : m->inst)
        brr_ctx_destroy(c);
    for (cudaEvent_t e : m->ready)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : m->ev)
        if (e)
            cudaEventDestroy(e);
    if (m->done)
        cudaEventDestroy(m->done);
    cudaFree(m->d_t);
    cudaFreeHost(m->h_t);
    if (m->exec)
        cudaGraphExecDestroy(m->exec);
    if (m->st)
        cudaStreamDestroy(m->st);
}

// Shared memory of an instance's sweep over G slices with round width B.
size_t inst_smem(const brr_ctx *c, int G, int B)
{
    const int64_t chunks = (c->cfg.N + kChunkInd - 1) / kChunkInd;
    const int64_t maxch = (chunks + G - 1) / G;
    SweepArgs a{};
    a.B = B;
    a.n_groups = c->cfg.n_groups;
    a.slice_max = (int)(maxch * kChunkInd);
    a.slot_bytes = (int)(maxch * 16);
    return sweep_smem_bytes(c->cfg.form, c->kind, a);
}

// Fewest CTAs whose slices fit the shared memory limit (0: none does).
int min_ctas(const brr_ctx *c, int B, size_t limit)
{
    const int64_t chunks = (c->cfg.N + kChunkInd - 1) / kChunkInd;
    for (int G = 1; G <= chunks && G <= 4096; ++G)
        if (inst_smem(c, G, B) <= limit && (c->kind != BRR_KIND_RAGGED || (chunks + G - 1) / G * kChunkInd <= 65536))
            return G;
    return 0;
}

// CTAs per instance: every instance gets its minimum, the rest go one at a
// time to the instance with the largest estimated time work_i / G_i.
bool allocate(const std::vector<double> &work, const std::vector<int> &mins, const std::vector<int> &maxs, int total,
              std::vector<int> &G)
{
    const int n = (int)work.size();
    G = mins;
    int used = 0;
    for (int g : G)
        used += g;
    if (used > total)
        return false;
    for (int left = total - used; left > 0; --left) {
        int best = -1;
        double bt = -1.0;
        for (int i = 0; i < n; ++i) {
            if (G[i] >= maxs[i])
                continue;
            const double t = work[i] / G[i];
            if (t > bt) {
                bt = t;
                best = i;
            }
        }
        if (best < 0)
            break;
        ++G[best];
    }
    return true;
}

// Ends a stream capture that failed part way, so the stream is usable again.
int abandon_capture(brr_multi *m, int rc)
{
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(m->st, &g);
    if (g)
        cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

// One iteration of every instance: the host parts of updateMu, then one CUDA
// graph holding all instances' draws, sweep orders, constants and records,
// the one launch of the multi-instance sweep, and all instances' statistics
// and read-backs; the graph is captured each iteration (the launch arguments
// carry the new updateMu shifts) and updated in place.
int run_iteration(brr_multi *m)
{
    const int n = m->n;
    std::vector<SweepArgs> args(n);
    std::vector<brr_sweep_out> so(n);
    std::vector<uint32_t> its(n);
    std::vector<double> et(n);
    for (int i = 0; i < n; ++i) {
        its[i] = m->inst[i]->iteration;
        const int rc = iter_pre_dev(*m->inst[i], its[i]);
        if (rc)
            return rc;
    }
    size_t smem = 0;
    MultiSweepArgs ma{};
    ma.n = n;
    ma.cta_start[0] = 0;
    for (int i = 0; i < n; ++i) {
        brr_ctx &c = *m->inst[i];
        MULTI_CUDA(cudaStreamSynchronize(c.st));
        double mu_new = 0.0;
        const int rc = iter_pre_host(c, its[i], mu_new, et[i]);
        if (rc)
            return rc;
        sweep_stage(&c);
        size_t si = 0;
        sweep_args(&c, mu_new, et[i], args[i], si);
        args[i].t_out = m->d_t + 2 * i;
        smem = std::max(smem, si);
        ma.cta_start[i + 1] = ma.cta_start[i] + c.G;
        ma.kind[i] = c.kind == BRR_KIND_DENSE ? 0 : 1;
        ma.inst[i] = args[i];
    }
    // occupancy check; also sets the kernel's shared-memory attribute outside the capture
    const int per_sm = sweep_multi_max_ctas_per_sm(m->form, m->kmax, smem);
    if (per_sm < 1 || (int64_t)per_sm * m->sms < ma.cta_start[n])
        return api_fail(BRR_ERR_ARG, "the instances need " + std::to_string(ma.cta_start[n]) +
                                         " co-resident CTAs with " + std::to_string(smem) + " bytes of shared memory");
    MULTI_CUDA(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < n; ++i) {
        brr_ctx &c = *m->inst[i];
        int rc = iter_enqueue_draws(c, its[i], m->st);
        if (!rc)
            rc = sweep_enqueue_inputs(&c, et[i], m->st);
        if (rc)
            return abandon_capture(m, rc);
    }
    cudaError_t e = launch_sweep_multi(m->form, m->kmax, ma, smem, m->st);
    if (e != cudaSuccess)
        return abandon_capture(m, api_fail(BRR_ERR_CUDA, std::string("multi-instance sweep: ") + cudaGetErrorString(e)));
    for (int i = 0; i < n; ++i) {
        const int rc = sweep_enqueue_outputs(m->inst[i], m->st);
        if (rc)
            return abandon_capture(m, rc);
    }
    e = cudaMemcpyAsync(m->h_t, m->d_t, sizeof(unsigned long long) * 2 * n, cudaMemcpyDeviceToHost, m->st);
    if (e != cudaSuccess)
        return abandon_capture(m, api_fail(BRR_ERR_CUDA, cudaGetErrorString(e)));
    cudaGraph_t graph = nullptr;
    MULTI_CUDA(cudaStreamEndCapture(m->st, &graph));
    if (m->exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(m->exec, graph, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(m->exec);
            m->exec = nullptr;
        }
    }
    if (!m->exec && (e = cudaGraphInstantiate(&m->exec, graph, 0)) != cudaSuccess) {
        cudaGraphDestroy(graph);
        m->exec = nullptr;
        return api_fail(BRR_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(e));
    }
    cudaGraphDestroy(graph);
    MULTI_CUDA(cudaEventRecord(m->ev[0], m->st));
    MULTI_CUDA(cudaGraphLaunch(m->exec, m->st));
    MULTI_CUDA(cudaEventRecord(m->ev[1], m->st));
    MULTI_CUDA(cudaStreamSynchronize(m->st));
    for (int i = 0; i < n; ++i) {
        brr_ctx &c = *m->inst[i];
        int rc = sweep_collect(&c, &so[i]);
        if (rc)
            return rc;
        rc = iter_post(c, so[i], its[i]);
        if (rc)
            return rc;
    }
    m->inst_ms.assign(n, 0.0);
    for (int i = 0; i < n; ++i)
        m->inst_ms[i] = m->h_t[2 * i + 1] >= m->h_t[2 * i] ? (double)(m->h_t[2 * i + 1] - m->h_t[2 * i]) / 1e6 : 0.0;
    float ms = 0.f;
    MULTI_CUDA(cudaEventElapsedTime(&ms, m->ev[0], m->ev[1]));
    m->last_sweep_ms += ms;
    return BRR_OK;
}

}  // namespace

extern "C" {

int brr_multi_create(const brr_config *cfgs, int32_t n, brr_multi **out)
{
    if (!cfgs || !out || n < 1 || n > kMaxInstances)
        return api_fail(BRR_ERR_ARG, "need 1 to 32 instance configurations");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (cfgs[i].form != cfgs[0].form || cfgs[i].device != cfgs[0].device)
            return api_fail(BRR_ERR_ARG, "all instances of a multi-instance run share the sweep form and the device");
        if (cfgs[i].kind != BRR_KIND_DENSE && cfgs[i].kind != BRR_KIND_RAGGED && cfgs[i].kind != BRR_KIND_EIGEN)
            return api_fail(BRR_ERR_ARG, "unknown marker kind");
        if (cfgs[i].async_batch != 0)
            return api_fail(BRR_ERR_ARG, "the multi-instance sweep runs the synchronous schedule");
        if (cfgs[i].cluster != 0)
            return api_fail(BRR_ERR_ARG, "the multi-instance sweep exchanges through L2, not as clusters");
    }
    brr_multi *m = new brr_multi();
    m->n = n;
    m->form = cfgs[0].form;
    m->dev = cfgs[0].device;
    auto bail = [&](int rc) {
        free_multi(m);
        delete m;
        return rc;
    };
    cudaDeviceProp prop;
    if (cudaSetDevice(m->dev) != cudaSuccess || cudaGetDeviceProperties(&prop, m->dev) != cudaSuccess)
        return bail(api_fail(BRR_ERR_DEVICE, "no usable device"));
    m->sms = prop.multiProcessorCount;
    // instances are created with a provisional slicing and sliced again once all are known
    for (int i = 0; i < n; ++i) {
        brr_config c = cfgs[i];
        c.grid = 0;
        c.gram = -1;
        c.pair_rounds = -1;
        brr_ctx *x = nullptr;
        const int rc = brr_ctx_create(&c, &x);
        if (rc)
            return bail(rc);
        m->inst.push_back(x);
        for (int g = 0; g < c.n_groups; ++g)
            m->kmax = std::max(m->kmax, c.K[g]);
    }
    // dynamic shared memory: what a CTA may use beside the kernel's static arrays
    m->smem_limit = prop.sharedMemPerBlockOptin - sweep_multi_static_smem(m->form, m->kmax);
    // first split of the SMs: at least what the slices need, the rest by N*M;
    // when the default round widths need more CTAs than there are SMs, every
    // instance starts at the narrowest width (the smallest code ring)
    std::vector<double> work(n);
    std::vector<int> mins(n), maxs(n), G, widths(n);
    const int narrowest = 8;
    for (int pass = 0; pass < 2; ++pass) {
        int need = 0;
        for (int i = 0; i < n; ++i) {
            const brr_ctx *c = m->inst[i];
            widths[i] = pass == 0 ? c->B : narrowest;
            work[i] = (double)c->cfg.N * (double)c->cfg.M;
            mins[i] = min_ctas(c, widths[i], m->smem_limit);
            maxs[i] = (int)((c->cfg.N + kChunkInd - 1) / kChunkInd);
            if (mins[i] == 0)
                return bail(api_fail(BRR_ERR_ARG, "instance " + std::to_string(i) + " does not fit shared memory"));
            need += mins[i];
        }
        if (need <= m->sms)
            break;
    }
    if (!allocate(work, mins, maxs, m->sms, G))
        return bail(api_fail(BRR_ERR_ARG, "the instances need more CTAs than the GPU has SMs"));
    for (int i = 0; i < n; ++i) {
        brr_ctx *c = m->inst[i];
        brr_config cf = c->cfg;
        brr_ctx_destroy(c);
        cf.grid = G[i];
        cf.spec_width = widths[i];
        brr_ctx *x = nullptr;
        const int rc = brr_ctx_create(&cf, &x);
        m->inst[i] = x;
        if (rc)
            return bail(rc);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        e = cudaEventCreate(&m->ev[i]);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&m->done, cudaEventDisableTiming);
    m->ready.assign(n, nullptr);
    for (int i = 0; i < n && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&m->ready[i], cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&m->d_t, sizeof(unsigned long long) * 2 * n);
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&m->h_t, sizeof(unsigned long long) * 2 * n);
    if (e != cudaSuccess)
        return bail(api_fail(BRR_ERR_CUDA, cudaGetErrorString(e)));
    *out = m;
    return BRR_OK;
}

int brr_multi_destroy(brr_multi *m)
{
    if (!m)
        return BRR_OK;
    cudaSetDevice(m->dev);
    free_multi(m);
    delete m;
    return BRR_OK;
}

int brr_multi_pack_bed(brr_multi *m, int32_t i, const uint8_t *bed, int64_t nbytes)
{
    if (!m || i < 0 || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    return brr_pack_bed(m->inst[i], bed, nbytes);
}

int brr_multi_pack_bed_device(brr_multi *m, int32_t i, const uint8_t *d_bed, int64_t nbytes)
{
    if (!m || i < 0 || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    return brr_pack_bed_device(m->inst[i], d_bed, nbytes);
}

int brr_multi_set_groups(brr_multi *m, int32_t i, const int32_t *group)
{
    if (!m || i < 0 || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    return brr_set_groups(m->inst[i], group);
}

int brr_multi_set_phenotype(brr_multi *m, int32_t i, const float *y)
{
    if (!m || i < 0 || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    return brr_set_phenotype(m->inst[i], y);
}

int brr_multi_init(brr_multi *m)
{
    if (!m)
        return api_fail(BRR_ERR_ARG, "null multi-instance handle");
    for (int i = 0; i < m->n; ++i) {
        const int rc = brr_init_chain(m->inst[i]);
        if (rc)
            return rc;
    }
    m->inited = true;
    return BRR_OK;
}

int brr_multi_iterate(brr_multi *m, int32_t n_iter)
{
    if (!m || !m->inited)
        return api_fail(BRR_ERR_ARG, "instances not initialised");
    MULTI_CUDA(cudaSetDevice(m->dev));
    const auto t0 = std::chrono::steady_clock::now();
    m->last_sweep_ms = 0.0;
    for (int32_t k = 0; k < n_iter; ++k) {
        const int rc = run_iteration(m);
        if (rc)
            return rc;
    }
    MULTI_CUDA(cudaDeviceSynchronize());
    m->last_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return BRR_OK;
}

// Autotuner: round width per instance from the candidates, then `rounds`
// rebalancing steps of the CTAs.  Every step is a real iteration of all chains.
int brr_multi_tune(brr_multi *m, int32_t rounds)
{
    if (!m || !m->inited || rounds < 0)
        return api_fail(BRR_ERR_ARG, "instances not initialised");
    MULTI_CUDA(cudaSetDevice(m->dev));
    const int n = m->n;
    const int cand[3] = {8, 16, 32};
    std::vector<double> best(n, 1e300);
    std::vector<int> bestB(n);
    for (int i = 0; i < n; ++i)
        bestB[i] = m->inst[i]->B;
    for (int b : cand) {
        for (int i = 0; i < n; ++i) {
            brr_ctx *c = m->inst[i];
            const int B = inst_smem(c, c->G, b) <= m->smem_limit ? b : c->B;
            const int rc = reslice(c, c->G, B);
            if (rc)
                return rc;
        }
        m->last_sweep_ms = 0.0;
        const int rc = run_iteration(m);
        if (rc)
            return rc;
        for (int i = 0; i < n; ++i)
            if (m->inst_ms[i] < best[i]) {
                best[i] = m->inst_ms[i];
                bestB[i] = m->inst[i]->B;
            }
    }
    for (int i = 0; i < n; ++i) {
        const int rc = reslice(m->inst[i], m->inst[i]->G, bestB[i]);
        if (rc)
            return rc;
    }
    for (int r = 0; r < rounds; ++r) {
        m->last_sweep_ms = 0.0;
        int rc = run_iteration(m);
        if (rc)
            return rc;
        std::vector<double> work(n);
        std::vector<int> mins(n), maxs(n), G;
        for (int i = 0; i < n; ++i) {
            brr_ctx *c = m->inst[i];
            work[i] = std::max(m->inst_ms[i], 1e-3) * c->G;
            mins[i] = min_ctas(c, c->B, m->smem_limit);
            maxs[i] = (int)((c->cfg.N + kChunkInd - 1) / kChunkInd);
        }
        if (!allocate(work, mins, maxs, m->sms, G))
            return api_fail(BRR_ERR_ARG, "the instances need more CTAs than the GPU has SMs");
        for (int i = 0; i < n; ++i) {
            if (G[i] == m->inst[i]->G)
                continue;
            rc = reslice(m->inst[i], G[i], 0);
            if (rc)
                return rc;
        }
    }
    return BRR_OK;
}

int brr_multi_get_state(brr_multi *m, int32_t i, brr_state *st)
{
    if (!m || i < 0 || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    return brr_get_state(m->inst[i], st);
}

// Wait limit and phantom barrier arrivals of instance i (every instance when
// i < 0): the instance's own context settings, read when its sweep arguments
// are built.
int brr_multi_set_wait_limit(brr_multi *m, int32_t i, uint64_t timeout_ns, int32_t phantom_arrivals)
{
    if (!m || i >= m->n)
        return api_fail(BRR_ERR_ARG, "instance out of range");
    for (int k = 0; k < m->n; ++k)
        if (i < 0 || k == i) {
            const int rc = brr_set_wait_limit(m->inst[k], timeout_ns, phantom_arrivals);
            if (rc)
                return rc;
        }
    return BRR_OK;
}

// Device time of the iteration graphs (all instances' draws, records, the one
// sweep launch and the statistics) and wall time of the last brr_multi_iterate
// call; per instance (optional, n values each): CTAs, round width and the last
// sweep's time on the device timer (ms).
int brr_multi_get_timing(brr_multi *m, double *sweep_ms, double *total_ms, int32_t *ctas, int32_t *width,
                         double *inst_ms)
{
    if (!m)
        return api_fail(BRR_ERR_ARG, "null multi-instance handle");
    if (sweep_ms)
        *sweep_ms = m->last_sweep_ms;
    if (total_ms)
        *total_ms = m->last_total_ms;
    for (int i = 0; i < m->n; ++i) {
        if (ctas)
            ctas[i] = m->inst[i]->G;
        if (width)
            width[i] = m->inst[i]->B;
        if (inst_ms)
            inst_ms[i] = i < (int)m->inst_ms.size() ? m->inst_ms[i] : 0.0;
    }
    return BRR_OK;
}

}  // extern "C"
