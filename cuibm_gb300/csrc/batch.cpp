// Batched instances: many independent cases advanced together on one GPU, on top
// of the single-case C ABI (no counterpart in the reference, which runs one case
// per process, src/cuIBM.cu:61-74).
//
// Why this shape on GB300: at the benchmark sizes (10^4..3x10^5 cells) a step is
// latency-bound - grid barriers of the persistent solves, short dependent phases -
// and one instance leaves most of the GPU idle.  Each instance here keeps its own
// stream and step graph, and its persistent solves are launched on a fraction of
// the SMs (-solverBlocks), so the cooperative solves of several instances are
// resident at once and the other instances' short kernels fill the gaps.  The
// instances never wait on one another: an instance that needs more iterations in a
// step delays only itself (a single launch stepping all instances in lockstep
// phases would hold every instance to the slowest one's iteration count).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cuibm.h"
#include "batch_member.h"

// With CUIBM_BATCH_GRAPH=1 the batch step is one CUDA graph: every instance's step graph
// is a child of it, with no edges between them (the instances are independent),
// launched once per batch step on the batch's own stream, and rebuilt when an
// instance's step graph changes (a new solver grid from the autotuner, an option).  It
// is off by default: on the 64-instance benchmark it ran at 208 Mcell-steps/s against
// 266 with every instance's step graph launched on the instance's own stream (the
// default).  Where an instance's steps need host work between them (see
// cuibm_batch_member_graph), the batch always steps the instances one by one.
struct cuibm_batch {
    std::vector<cuibm_ctx *> ctx;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraph_t> members;  // the instance graphs the batch graph was built from
};

static void drop_graph(cuibm_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->members.clear();
}

// the batch step graph for the instances' current step graphs; false where one of them
// has none (the batch then steps the instances one by one)
static bool batch_graph(cuibm_batch *b)
{
    std::vector<cudaGraph_t> cur(b->ctx.size());
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        cur[k] = cuibm_batch_member_graph(b->ctx[k]);
        if (!cur[k]) {
            drop_graph(b);
            return false;
        }
    }
    if (b->exec && cur == b->members) return true;
    drop_graph(b);
    if (!b->stream && cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaGraphCreate(&b->graph, 0) != cudaSuccess) return false;
    for (cudaGraph_t g : cur) {
        cudaGraphNode_t node;
        if (cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, g) != cudaSuccess) {
            drop_graph(b);
            return false;
        }
    }
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
        drop_graph(b);
        return false;
    }
    b->members = cur;
    return true;
}

static std::string g_batch_create_error;

static int batch_fail(cuibm_batch *b, int code, const std::string &msg)
{
    if (b) b->err = msg;
    else g_batch_create_error = msg;
    return code;
}

extern "C" {

int cuibm_batch_create(int n, const char *const *case_folders, int argc, const char **argv, int solver_blocks,
                       cuibm_batch **out)
{
    if (!out || n <= 0 || !case_folders) return batch_fail(nullptr, CUIBM_ERR_BAD_INPUT, "batch: no cases");
    *out = nullptr;
    int blocks = solver_blocks;
    if (blocks <= 0) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return batch_fail(nullptr, CUIBM_ERR_CUDA, "batch: cannot query the device");
        // a quarter of the SMs, with the solves built for two blocks per SM: on the
        // 64-instance benchmark 38 blocks gave 176 Mcell-steps/s, 19 blocks 172 and 12
        // blocks 142 (built for one block per SM: 136, 152 and 143)
        blocks = sms / 4 > 0 ? sms / 4 : 1;
    }
    const std::string nb = std::to_string(blocks);
    std::vector<const char *> args(argv, argv + (argc > 0 ? argc : 0));
    args.push_back("-solverBlocks");
    args.push_back(nb.c_str());
    args.push_back("-solverPack");  // two instances' solve blocks may share an SM
    args.push_back("2");
    cuibm_batch *b = new cuibm_batch();
    for (int k = 0; k < n; ++k) {
        cuibm_ctx *c = nullptr;
        const int st = cuibm_create(case_folders[k], (int)args.size(), args.data(), &c);
        if (st != CUIBM_OK) {
            const std::string msg = "batch: instance " + std::to_string(k) + " (" + case_folders[k] +
                                    "): " + cuibm_last_error(nullptr);
            cuibm_batch_destroy(b);
            return batch_fail(nullptr, st, msg);
        }
        b->ctx.push_back(c);
    }
    *out = b;
    return CUIBM_OK;
}

int cuibm_batch_initialise(cuibm_batch *b)
{
    if (!b) return CUIBM_ERR_STATE;
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        const int st = cuibm_initialise(b->ctx[k]);
        if (st != CUIBM_OK)
            return batch_fail(b, st, "batch: instance " + std::to_string(k) + ": " + cuibm_last_error(b->ctx[k]));
        // steps are enqueued without waiting; cuibm_batch_step checks them at its end
        cuibm_set_option(b->ctx[k], "step_sync", 0);
    }
    return CUIBM_OK;
}

int cuibm_batch_step(cuibm_batch *b, int nsteps)
{
    if (!b) return CUIBM_ERR_STATE;
    if (nsteps < 0) return batch_fail(b, CUIBM_ERR_BAD_INPUT, "batch: nsteps < 0");
    const char *eg = getenv("CUIBM_BATCH_GRAPH");
    if (nsteps > 0 && eg && eg[0] == '1' && batch_graph(b)) {
        // the instances' own streams may hold work enqueued before (initialisation,
        // field writes): the batch stream starts after it
        for (cuibm_ctx *c : b->ctx)
            if (cudaStreamSynchronize(cuibm_batch_member_stream(c)) != cudaSuccess)
                return batch_fail(b, CUIBM_ERR_CUDA, "batch: an instance's stream failed");
        for (int s = 0; s < nsteps; ++s)
            if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess)
                return batch_fail(b, CUIBM_ERR_CUDA, "batch: the batch step graph did not launch");
        if (cudaStreamSynchronize(b->stream) != cudaSuccess)
            return batch_fail(b, CUIBM_ERR_CUDA, "batch: the batch step graph failed");
        for (cuibm_ctx *c : b->ctx) cuibm_batch_member_advance(c, nsteps);
    } else {
        for (int s = 0; s < nsteps; ++s)
            for (size_t k = 0; k < b->ctx.size(); ++k) {
                const int st = cuibm_step(b->ctx[k], 1);
                if (st != CUIBM_OK)
                    return batch_fail(b, st,
                                      "batch: instance " + std::to_string(k) + ": " + cuibm_last_error(b->ctx[k]));
            }
    }
    int first = CUIBM_OK;
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        const int st = cuibm_step(b->ctx[k], 0);  // waits for the instance and checks its solves
        if (st != CUIBM_OK && first == CUIBM_OK) {
            first = st;
            batch_fail(b, st, "batch: instance " + std::to_string(k) + ": " + cuibm_last_error(b->ctx[k]));
        }
    }
    return first;
}

// The best grid depends on the instances' sizes and count (fewer, larger blocks give
// each solve more of the GPU; more, smaller shares let more solves run at once), so
// it is measured on the batch itself.  Candidates: one block count for every instance
// (a quarter, sixth or eighth of the SMs), or a count per instance from its pressure
// unknowns at 6, 8, 12, 16 or 24 rows a thread (512 threads a block; at least 2 blocks,
// at most half the SMs): at 16 rows a thread a 9k-cell cavity takes 2 blocks and a
// 262k-cell one 32.
int cuibm_batch_autotune(cuibm_batch *b, int steps, int *blocks_out)
{
    if (!b) return CUIBM_ERR_STATE;
    if (steps <= 0) return batch_fail(b, CUIBM_ERR_BAD_INPUT, "batch: autotune needs steps > 0");
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return batch_fail(b, CUIBM_ERR_CUDA, "batch: cannot query the device");
    std::vector<int> cand;  // > 0: blocks for every instance; < 0: minus the rows a thread
    for (int d : {4, 6, 8}) {
        const int nb = sms / d > 0 ? sms / d : 1;
        if (cand.empty() || cand.back() != nb) cand.push_back(nb);
    }
    for (int r : {6, 8, 12, 16, 24}) cand.push_back(-r);
    std::vector<int> rows(b->ctx.size(), 1);
    for (size_t k = 0; k < b->ctx.size(); ++k) {
        cuibm_info info;
        if (cuibm_get_info(b->ctx[k], &info) == CUIBM_OK) rows[k] = info.numP;
    }
    const int most = sms / 2 > 2 ? sms / 2 : 2;
    auto use = [&](int c) {
        for (size_t k = 0; k < b->ctx.size(); ++k) {
            int nb = c;
            if (c < 0) {
                const long per = 512L * -c;
                nb = (int)((rows[k] + per - 1) / per);
                nb = nb < 2 ? 2 : (nb > most ? most : nb);
            }
            const int st = cuibm_set_option(b->ctx[k], "solver_blocks", nb);
            if (st != CUIBM_OK)
                return batch_fail(b, st, "batch: instance " + std::to_string(k) + ": " + cuibm_last_error(b->ctx[k]));
        }
        return (int)CUIBM_OK;
    };
    std::vector<double> t(cand.size(), 0.0);
    for (int pass = 0; pass < 2; ++pass)
        for (size_t q = 0; q < cand.size(); ++q) {
            const size_t k = pass == 0 ? q : cand.size() - 1 - q;
            int st = use(cand[k]);
            if (st != CUIBM_OK) return st;
            const auto t0 = std::chrono::steady_clock::now();
            st = cuibm_batch_step(b, steps);  // returns after every instance finished
            if (st != CUIBM_OK) return st;
            t[k] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    size_t best = 0;
    for (size_t k = 1; k < cand.size(); ++k)
        if (t[k] < t[best]) best = k;
    const int st = use(cand[best]);
    if (st != CUIBM_OK) return st;
    if (blocks_out) *blocks_out = cand[best];
    return CUIBM_OK;
}

int cuibm_batch_size(const cuibm_batch *b) { return b ? (int)b->ctx.size() : 0; }

cuibm_ctx *cuibm_batch_instance(cuibm_batch *b, int k)
{
    return (b && k >= 0 && k < (int)b->ctx.size()) ? b->ctx[k] : nullptr;
}

const char *cuibm_batch_error(const cuibm_batch *b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

void cuibm_batch_destroy(cuibm_batch *b)
{
    if (!b) return;
    drop_graph(b);
    if (b->stream) cudaStreamDestroy(b->stream);
    for (cuibm_ctx *c : b->ctx) cuibm_destroy(c);
    delete b;
}

}  // extern "C"
