// Minimal stand-in for the glog API surface Puck's sources use (LOG, CHECK,
// InitGoogleLogging, SetLogDestination). INFO lines are dropped unless the
// environment variable PUCK_SHIM_LOG is set; ERROR lines go to stderr; FATAL
// aborts, as glog does. Test infrastructure only.
#pragma once
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace shimlog {
enum Severity { INFO = 0, WARNING = 1, ERROR = 2, FATAL = 3 };
bool info_enabled();
class Line {
public:
    Line(int sev, const char* file, int line) : _sev(sev) {
        _os << "[puck-ref " << "IWEF"[sev] << "] " << file << ":" << line << " ";
    }
    ~Line() {
        if (_sev >= ERROR || info_enabled()) {
            std::cerr << _os.str() << std::endl;
        }
        if (_sev == FATAL) {
            std::abort();
        }
    }
    std::ostream& stream() { return _os; }

private:
    int _sev;
    std::ostringstream _os;
};
}  // namespace shimlog

#define LOG(sev) ::shimlog::Line(::shimlog::sev, __FILE__, __LINE__).stream()
#define CHECK(cond) \
    if (!(cond)) ::shimlog::Line(::shimlog::FATAL, __FILE__, __LINE__).stream() << "CHECK failed: " #cond " "

namespace google {
void InitGoogleLogging(const char* argv0);
void SetLogDestination(int severity, const char* base_filename);
}  // namespace google
