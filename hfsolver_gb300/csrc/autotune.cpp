// Autotuner for the quartet-tile shapes of the ERI and Fock-digest kernels.
//
// The shape knobs are, per quartet class:
//   * ERI: primitive quartets per lane before a quartet's primitive loop is
//     split over more lanes (the `split` of each segment),
//   * digest: lanes per quartet in the Fock build.
// With tuning on (hfgpu_options.autotune or HFGPU_AUTOTUNE=1), the first time a
// (kernel, class, size bucket) is met its candidates are timed on the real
// launch and the fastest is kept in a process-wide table; later molecules of
// the same bucket reuse it.  With tuning off, the built-in rules are used.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "autotune.h"

namespace hfgpu {

namespace {
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int>, int> g_table;  // (kind, tb, tk, bucket) -> choice
}  // namespace

bool tune_env_enabled()
{
    const char* e = std::getenv("HFGPU_AUTOTUNE");
    return e && e[0] && e[0] != '0';
}

int tune_bucket(int64_t nq)
{
    int b = 0;
    while (nq > 1) {
        nq >>= 1;
        ++b;
    }
    return b;
}

bool tune_get(TuneKind kind, int tb, int tk, int bucket, int* choice)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_table.find({(int)kind, tb, tk, bucket});
    if (it == g_table.end()) return false;
    *choice = it->second;
    return true;
}

void tune_set(TuneKind kind, int tb, int tk, int bucket, int choice)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_table[{(int)kind, tb, tk, bucket}] = choice;
}

void tune_clear()
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_table.clear();
}

std::string tune_dump()
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    std::string s;
    char line[96];
    for (auto& e : g_table) {
        std::snprintf(line, sizeof line, "%s %d %d %d %d\n", std::get<0>(e.first) == TUNE_ERI ? "eri" : "digest",
                      std::get<1>(e.first), std::get<2>(e.first), std::get<3>(e.first), e.second);
        s += line;
    }
    return s;
}

}  // namespace hfgpu
