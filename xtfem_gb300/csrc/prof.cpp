// prof.cpp -- CUDA-event timing of kernel classes on the launching stream.
//
// When enabled, every launch of a timed class is bracketed by two events
// recorded on the stream the kernel runs on; the elapsed times are summed
// when read (after a synchronize).  Used by bench.py to report the average
// duration of the dominant kernel inside the timed region.
#include "prof.h"

#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/xtfem_gb300_host.h"
#include "solver.h"
#include "xt_device.h"

namespace xt {

namespace {
// Records are keyed by token so that several host threads (independent
// systems on their own streams) can time kernels at once.
struct Rec {
    int cls;
    cudaEvent_t a, b;
    bool ended;
    double bytes;
};
std::mutex g_mu;
bool g_on = false;
int g_next = 0;
std::map<int, Rec> g_open;
std::vector<cudaEvent_t> g_pool;
long long g_count[PROF_NCLASS] = {0};
double g_ms[PROF_NCLASS] = {0};
double g_bytes[PROF_NCLASS] = {0};

cudaEvent_t take()
{
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Sum finished records (caller holds g_mu).
void settle_locked()
{
    for (auto it = g_open.begin(); it != g_open.end();) {
        Rec& r = it->second;
        if (!r.ended) { ++it; continue; }
        cudaEventSynchronize(r.b);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            g_count[r.cls] += 1;
            g_ms[r.cls] += ms;
            g_bytes[r.cls] += r.bytes;
        }
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
        it = g_open.erase(it);
    }
}

void settle()
{
    std::lock_guard<std::mutex> lk(g_mu);
    settle_locked();
}
}  // namespace

int prof_begin(int cls, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_on) return -1;
    if (g_open.size() > 4096) settle_locked();
    const int id = g_next++ & 0x3fffffff;
    Rec r{cls, take(), take(), false, 0.0};
    cudaEventRecord(r.a, s);
    g_open[id] = r;
    return id;
}

void prof_end(int token, cudaStream_t s)
{
    if (token < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_open.find(token);
    if (it == g_open.end()) return;
    cudaEventRecord(it->second.b, s);
    it->second.ended = true;
}

void prof_cancel(int token)
{
    if (token < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_open.find(token);
    if (it == g_open.end()) return;
    // the events may still be pending on the stream: wait before reusing them
    if (it->second.ended) cudaEventSynchronize(it->second.b);
    g_pool.push_back(it->second.a);
    g_pool.push_back(it->second.b);
    g_open.erase(it);
}

void prof_bytes(int token, double bytes)
{
    if (token < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_open.find(token);
    if (it != g_open.end()) it->second.bytes += bytes;
}

}  // namespace xt

extern "C" {

int xt_profile(int enable)
{
    xt::settle();
    std::lock_guard<std::mutex> lk(xt::g_mu);
    xt::g_on = enable != 0;
    for (int c = 0; c < xt::PROF_NCLASS; ++c) {
        xt::g_count[c] = 0;
        xt::g_ms[c] = 0.0;
        xt::g_bytes[c] = 0.0;
    }
    return XT_OK;
}

int xt_profile_read(int cls, long long* count, double* ms)
{
    if (cls < 0 || cls >= xt::PROF_NCLASS) return XT_ERR_ARG;
    xt::settle();
    std::lock_guard<std::mutex> lk(xt::g_mu);
    if (count) *count = xt::g_count[cls];
    if (ms) *ms = xt::g_ms[cls];
    return XT_OK;
}

int xt_profile_bytes(int cls, double* bytes)
{
    if (cls < 0 || cls >= xt::PROF_NCLASS || !bytes) return XT_ERR_ARG;
    xt::settle();
    std::lock_guard<std::mutex> lk(xt::g_mu);
    *bytes = xt::g_bytes[cls];
    return XT_OK;
}

}  // extern "C"

// ------------------------------------------------ launch count and timers
namespace xt {
namespace {
std::atomic<long long> g_launches{0};
cudaEvent_t g_marks[8] = {nullptr};
}  // namespace

void note_launches(int n) { g_launches += n; }

void trace(const char* what)
{
    static int on = -1;
    if (on < 0) on = std::getenv("XTFEM_TRACE") ? 1 : 0;
    if (!on) return;
    cudaError_t e = cudaDeviceSynchronize();
    std::fprintf(stderr, "[xtfem] %s: %s\n", what, cudaGetErrorString(e));
    std::fflush(stderr);
}

}  // namespace xt

extern "C" {

long long xt_launch_count(void) { return xt::g_launches; }

int xt_mark(int slot)
{
    if (slot < 0 || slot >= 8) return XT_ERR_ARG;
    if (xt::ensure_init() != XT_OK) return XT_ERR_CUDA;
    if (!xt::g_marks[slot] && cudaEventCreate(&xt::g_marks[slot]) != cudaSuccess) return XT_ERR_CUDA;
    return cudaEventRecord(xt::g_marks[slot], xt::ctx().stream) == cudaSuccess ? XT_OK : XT_ERR_CUDA;
}

double xt_elapsed_ms(int a, int b)
{
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !xt::g_marks[a] || !xt::g_marks[b]) return -1.0;
    if (cudaEventSynchronize(xt::g_marks[b]) != cudaSuccess) return -1.0;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, xt::g_marks[a], xt::g_marks[b]) != cudaSuccess) return -1.0;
    return ms;
}

int xt_sync(void)
{
    if (!xt::ctx().ready) return XT_OK;
    return cudaDeviceSynchronize() == cudaSuccess ? XT_OK : XT_ERR_CUDA;
}

}  // extern "C"
