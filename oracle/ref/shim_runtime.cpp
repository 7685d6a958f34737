// Flag registry and logging hooks behind the gflags/glog stand-in headers.
// Test infrastructure only: it lets the reference's own sources build and run
// as the oracle.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "gflags/gflags.h"
#include "glog/logging.h"

namespace shimflags {
namespace {
struct Entry {
    void* ptr;
    Kind kind;
    bool modified;
};
std::map<std::string, Entry>& registry() {
    static std::map<std::string, Entry> r;
    return r;
}
std::mutex& registry_mutex() {
    static std::mutex m;
    return m;
}
std::string to_string(const Entry& e) {
    switch (e.kind) {
    case kInt32: return std::to_string(*static_cast<int32_t*>(e.ptr));
    case kBool: return *static_cast<bool*>(e.ptr) ? "true" : "false";
    case kDouble: return std::to_string(*static_cast<double*>(e.ptr));
    default: return *static_cast<std::string*>(e.ptr);
    }
}
}  // namespace

Registrar::Registrar(const char* name, void* ptr, Kind kind) {
    std::lock_guard<std::mutex> g(registry_mutex());
    registry()[name] = Entry{ptr, kind, false};
}

bool set_flag(const char* name, const char* value) {
    std::lock_guard<std::mutex> g(registry_mutex());
    auto it = registry().find(name);
    if (it == registry().end() || value == nullptr) {
        return false;
    }
    Entry& e = it->second;
    switch (e.kind) {
    case kInt32: *static_cast<int32_t*>(e.ptr) = (int32_t)std::strtol(value, nullptr, 10); break;
    case kBool:
        *static_cast<bool*>(e.ptr) =
            (std::strcmp(value, "true") == 0 || std::strcmp(value, "1") == 0 ||
             std::strcmp(value, "True") == 0);
        break;
    case kDouble: *static_cast<double*>(e.ptr) = std::strtod(value, nullptr); break;
    default: *static_cast<std::string*>(e.ptr) = value; break;
    }
    e.modified = true;
    return true;
}

bool get_flag(const char* name, std::string* value, bool* is_default) {
    std::lock_guard<std::mutex> g(registry_mutex());
    auto it = registry().find(name);
    if (it == registry().end()) {
        return false;
    }
    *value = to_string(it->second);
    *is_default = !it->second.modified;
    return true;
}
}  // namespace shimflags

namespace google {
std::string SetCommandLineOption(const char* name, const char* value) {
    if (!shimflags::set_flag(name, value)) {
        return std::string();
    }
    return std::string(name) + " set to " + value + "\n";
}

bool GetCommandLineFlagInfo(const char* name, CommandLineFlagInfo* info) {
    std::string v;
    bool is_default = true;
    if (!shimflags::get_flag(name, &v, &is_default)) {
        return false;
    }
    info->name = name;
    info->current_value = v;
    info->is_default = is_default;
    return true;
}

uint32_t ParseCommandLineFlags(int* argc, char*** argv, bool remove_flags) {
    (void)remove_flags;
    for (int i = 1; i < *argc; ++i) {
        const char* a = (*argv)[i];
        while (*a == '-') ++a;
        const char* eq = std::strchr(a, '=');
        if (eq == nullptr) continue;
        std::string key(a, eq - a);
        shimflags::set_flag(key.c_str(), eq + 1);
    }
    return 1;
}

void InitGoogleLogging(const char*) {}
void SetLogDestination(int, const char*) {}
}  // namespace google

namespace shimlog {
bool info_enabled() {
    static const bool on = std::getenv("PUCK_SHIM_LOG") != nullptr;
    return on;
}
}  // namespace shimlog
