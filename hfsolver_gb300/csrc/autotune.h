// Process-wide table of tuned kernel shapes (autotune.cpp).
#pragma once
#include <cstdint>
#include <string>

namespace hfgpu {

enum TuneKind { TUNE_ERI = 0, TUNE_DIGEST = 1 };

bool tune_env_enabled();        // HFGPU_AUTOTUNE=1 in the environment
int tune_bucket(int64_t nq);    // size bucket: floor(log2(quartets of the class))
bool tune_get(TuneKind kind, int tb, int tk, int bucket, int* choice);
void tune_set(TuneKind kind, int tb, int tk, int bucket, int choice);
void tune_clear();
// one line per entry: "<eri|digest> <bra type> <ket type> <bucket> <choice>"
std::string tune_dump();

}  // namespace hfgpu
