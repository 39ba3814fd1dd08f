// tune_cache.h — the autotuners' JSON cache files (orn_batch_tune,
// orn_wave_tune): one object per tuned workload, keyed by a string naming
// the device and the workload, holding the chosen launch parameters as
// integers and the measured time:
//
//   {
//     "<key>": {"<name>": <int>, ..., "ms": <float>},
//     ...
//   }
//
// Host code only.  The reader is deliberately small: it accepts what the
// writer produces (and hand edits of the numbers); an entry missing a field
// the caller asks for is skipped by the caller, which then tunes that
// workload again.
#pragma once

#include <map>
#include <string>
#include <vector>

namespace orn {

struct TuneEntry {
    std::map<std::string, long> fields;   // integer launch parameters
    double ms = 0.0;                      // the chosen configuration's time
};

// The entries of the file at `path` (empty when it is missing or unreadable).
std::map<std::string, TuneEntry> read_tune_cache(const char* path);

// Writes `entries` to `path` (through a temporary file renamed over it),
// each with its own integer fields, those in `names` first and in that
// order; false on an I/O error.
bool write_tune_cache(const char* path, const std::map<std::string, TuneEntry>& entries,
                      const std::vector<std::string>& names);

}  // namespace orn
