// Tuning parameters (block sizes, panel cluster size, tile shapes) with
// built-in defaults, overridable through ddla_tune_set -- the hook the
// autotuner (ddla_gb300/autotune.py) writes its chosen values through.
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "common.cuh"

namespace ddla {
namespace {
std::mutex g_mu;
std::map<std::string, int64_t> &table() {
    static std::map<std::string, int64_t> t;
    return t;
}
}  // namespace

int64_t tune_get(const char *key, int64_t dflt) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = table().find(key);
    return it == table().end() ? dflt : it->second;
}

}  // namespace ddla

using namespace ddla;

extern "C" int ddla_tune_set(const char *key, int64_t value) {
    if (!key || !*key) return -1;
    std::lock_guard<std::mutex> g(g_mu);
    if (value == INT64_MIN) table().erase(key);
    else table()[key] = value;
    return 0;
}

extern "C" int64_t ddla_tune_get(const char *key, int64_t dflt) { return key ? tune_get(key, dflt) : dflt; }
