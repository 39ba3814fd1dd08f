// tune_cache.cpp — reading and writing the autotuners' JSON cache files
// (tune_cache.h).
#include "tune_cache.h"

#include <cstdio>
#include <cstdlib>

namespace orn {

std::map<std::string, TuneEntry> read_tune_cache(const char* path) {
    std::map<std::string, TuneEntry> out;
    if (!path) return out;
    FILE* f = std::fopen(path, "rb");
    if (!f) return out;
    std::string s;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
    std::fclose(f);
    size_t pos = 0;
    while ((pos = s.find('"', pos)) != std::string::npos) {
        const size_t kend = s.find('"', pos + 1);
        if (kend == std::string::npos) break;
        const std::string key = s.substr(pos + 1, kend - pos - 1);
        const size_t ob = s.find_first_not_of(" \t\r\n:", kend + 1);
        if (ob == std::string::npos || s[ob] != '{') {
            pos = kend + 1;
            continue;
        }
        const size_t cb = s.find('}', ob);
        if (cb == std::string::npos) break;
        // "name": number pairs inside the object
        TuneEntry e;
        size_t q = ob + 1;
        while (q < cb) {
            const size_t n0 = s.find('"', q);
            if (n0 == std::string::npos || n0 >= cb) break;
            const size_t n1 = s.find('"', n0 + 1);
            if (n1 == std::string::npos || n1 >= cb) break;
            const std::string name = s.substr(n0 + 1, n1 - n0 - 1);
            const size_t colon = s.find(':', n1);
            if (colon == std::string::npos || colon >= cb) break;
            const char* num = s.c_str() + colon + 1;
            char* end = nullptr;
            if (name == "ms") {
                e.ms = std::strtod(num, &end);
            } else {
                const long v = std::strtol(num, &end, 10);
                if (end != num) e.fields[name] = v;
            }
            q = (end && end > num) ? (size_t)(end - s.c_str()) : colon + 1;
        }
        out[key] = e;
        pos = cb + 1;
    }
    return out;
}

bool write_tune_cache(const char* path, const std::map<std::string, TuneEntry>& entries,
                      const std::vector<std::string>& names) {
    if (!path) return false;
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "{\n");
    size_t i = 0;
    for (const auto& kv : entries) {
        // each entry's own fields (a file may hold both tuners' entries):
        // those named in `names` first, in that order, then the rest
        std::fprintf(f, "  \"%s\": {", kv.first.c_str());
        const auto& fields = kv.second.fields;
        for (const auto& name : names) {
            auto it = fields.find(name);
            if (it != fields.end()) std::fprintf(f, "\"%s\": %ld, ", name.c_str(), it->second);
        }
        for (const auto& fv : fields) {
            bool listed = false;
            for (const auto& name : names) listed = listed || name == fv.first;
            if (!listed) std::fprintf(f, "\"%s\": %ld, ", fv.first.c_str(), fv.second);
        }
        std::fprintf(f, "\"ms\": %.3f}%s\n", kv.second.ms, ++i < entries.size() ? "," : "");
    }
    std::fprintf(f, "}\n");
    const bool ok = std::fclose(f) == 0;
    return ok && std::rename(tmp.c_str(), path) == 0;
}

}  // namespace orn
