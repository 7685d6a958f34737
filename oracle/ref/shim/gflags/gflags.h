// Minimal stand-in for the gflags API surface that Puck's sources use, so the
// reference search/train/build code compiles without the gflags library.
// Test infrastructure only (it builds the oracle copy of the reference).
//
// Supported: DEFINE_/DECLARE_{int32,bool,double,string},
// google::SetCommandLineOption, google::GetCommandLineFlagInfo (with
// CommandLineFlagInfo::is_default), google::ParseCommandLineFlags.
#pragma once
#include <cstdint>
#include <string>

namespace shimflags {
enum Kind { kInt32, kBool, kDouble, kString };
struct Registrar {
    Registrar(const char* name, void* ptr, Kind kind);
};
bool set_flag(const char* name, const char* value);
bool get_flag(const char* name, std::string* value, bool* is_default);
}  // namespace shimflags

namespace google {
struct CommandLineFlagInfo {
    std::string name;
    std::string current_value;
    bool is_default = true;
};
std::string SetCommandLineOption(const char* name, const char* value);
bool GetCommandLineFlagInfo(const char* name, CommandLineFlagInfo* info);
uint32_t ParseCommandLineFlags(int* argc, char*** argv, bool remove_flags);
}  // namespace google
namespace gflags = google;

#define SHIM_DEFINE_FLAG(type, kind, name, value)                                   \
    type FLAGS_##name = (value);                                                    \
    static ::shimflags::Registrar shim_flag_registrar_##name(#name, &FLAGS_##name, \
                                                             ::shimflags::kind)

#define DEFINE_int32(name, value, help) SHIM_DEFINE_FLAG(int32_t, kInt32, name, value)
#define DEFINE_bool(name, value, help) SHIM_DEFINE_FLAG(bool, kBool, name, value)
#define DEFINE_double(name, value, help) SHIM_DEFINE_FLAG(double, kDouble, name, value)
#define DEFINE_string(name, value, help) SHIM_DEFINE_FLAG(std::string, kString, name, value)

#define DECLARE_int32(name) extern int32_t FLAGS_##name
#define DECLARE_bool(name) extern bool FLAGS_##name
#define DECLARE_double(name) extern double FLAGS_##name
#define DECLARE_string(name) extern std::string FLAGS_##name
