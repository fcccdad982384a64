// Minimal stand-in for glog, used only to compile the reference headers into
// the test oracle (glog is not installed in this image). CHECK failures abort;
// LOG output goes to stderr and is discarded below WARNING.
#pragma once
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace saqg_shim {
struct NullStream {
    template <class T> NullStream &operator<<(const T &) { return *this; }
    NullStream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
struct FatalStream {
    std::ostringstream os;
    FatalStream(const char *file, int line, const char *what) { os << file << ":" << line << " CHECK failed: " << what << " "; }
    template <class T> FatalStream &operator<<(const T &v) { os << v; return *this; }
    FatalStream &operator<<(std::ostream &(*f)(std::ostream &)) { f(os); return *this; }
    [[noreturn]] ~FatalStream() { std::cerr << os.str() << std::endl; std::abort(); }
};
struct LogStream {
    bool on;
    explicit LogStream(bool o) : on(o) {}
    template <class T> LogStream &operator<<(const T &v) { if (on) std::cerr << v; return *this; }
    LogStream &operator<<(std::ostream &(*f)(std::ostream &)) { if (on) f(std::cerr); return *this; }
    ~LogStream() { if (on) std::cerr << std::endl; }
};
inline bool log_verbose() { static bool v = std::getenv("SAQG_REF_VERBOSE") != nullptr; return v; }
} // namespace saqg_shim

#define SAQG_SHIM_CHECK(cond, txt) \
    if (cond) {} else saqg_shim::FatalStream(__FILE__, __LINE__, txt)
#define CHECK(c) SAQG_SHIM_CHECK((c), #c)
#define CHECK_EQ(a, b) SAQG_SHIM_CHECK((a) == (b), #a " == " #b)
#define CHECK_NE(a, b) SAQG_SHIM_CHECK((a) != (b), #a " != " #b)
#define CHECK_LE(a, b) SAQG_SHIM_CHECK((a) <= (b), #a " <= " #b)
#define CHECK_LT(a, b) SAQG_SHIM_CHECK((a) < (b), #a " < " #b)
#define CHECK_GE(a, b) SAQG_SHIM_CHECK((a) >= (b), #a " >= " #b)
#define CHECK_GT(a, b) SAQG_SHIM_CHECK((a) > (b), #a " > " #b)
#define DCHECK(c) while (false) saqg_shim::NullStream()
#define DCHECK_EQ(a, b) while (false) saqg_shim::NullStream()
#define DCHECK_NE(a, b) while (false) saqg_shim::NullStream()
#define DCHECK_LE(a, b) while (false) saqg_shim::NullStream()
#define DCHECK_LT(a, b) while (false) saqg_shim::NullStream()
#define DCHECK_GE(a, b) while (false) saqg_shim::NullStream()
#define DCHECK_GT(a, b) while (false) saqg_shim::NullStream()
#define SAQG_SEV_INFO 0
#define SAQG_SEV_WARNING 1
#define SAQG_SEV_ERROR 2
#define LOG(sev) saqg_shim::LogStream(SAQG_SEV_##sev >= 1 || saqg_shim::log_verbose())
#define LOG_IF(sev, cond) saqg_shim::LogStream((cond) && (SAQG_SEV_##sev >= 1 || saqg_shim::log_verbose()))
