// isp_tuning.cpp - the launch-tuning table of the two streamed kernels (imop_tuning_set / _get):
// per (kernel, input format, width class) whether frames take the kernel at all, the rows of a band
// and the streaming kernel's segment size.  The tuner (imop_gb300/tuning.py) measures the entries on
// the device and stores them as JSON; the Python package loads its table at import.

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "imop_isp.h"
#include "isp_context.h"
#include "isp_kernels.h"

namespace imop {
namespace {

std::mutex g_tune_mu;
std::vector<ImopTuneEntry> g_tune;
std::atomic<int> g_tune_gen{0};

}  // namespace

TuneParams tuning_for(int kernel, int fmt, int width) {
    TuneParams t{true, kernel == IMOP_KERNEL_LITE ? 16 : 32, 100};
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (const ImopTuneEntry& e : g_tune) {
        if (e.kernel != kernel || (e.fmt != -1 && e.fmt != fmt) || width > e.max_width) continue;
        t.enabled = e.enabled != 0;
        t.band_rows = e.band_rows;
        t.seg_percent = e.seg_percent;
        break;
    }
    return t;
}

int tuning_generation() { return g_tune_gen.load(std::memory_order_relaxed); }

}  // namespace imop

using namespace imop;

extern "C" int imop_tuning_set(const ImopTuneEntry* entries, int n) {
    if (n < 0) return set_error(IMOP_ERR_INVALID_ARGUMENT, "negative entry count");
    if (n > 0 && !entries) return set_error(IMOP_ERR_NULL_INPUT, "entries is null");
    for (int i = 0; i < n; i++) {
        const ImopTuneEntry& e = entries[i];
        if ((e.kernel != IMOP_KERNEL_LITE && e.kernel != IMOP_KERNEL_STREAM) || e.fmt < -1 || e.fmt > 3 ||
            e.max_width < 1 || e.band_rows < 4 || e.band_rows > 1024 || e.seg_percent < 10 || e.seg_percent > 1000)
            return set_error(IMOP_ERR_INVALID_ARGUMENT, "tuning entry out of range");
    }
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.assign(entries, entries + n);
    g_tune_gen.fetch_add(1, std::memory_order_relaxed);
    return IMOP_OK;
}

extern "C" int imop_tuning_get(ImopTuneEntry* out, int cap) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (out)
        for (int i = 0; i < cap && i < (int)g_tune.size(); i++) out[i] = g_tune[i];
    return (int)g_tune.size();
}
