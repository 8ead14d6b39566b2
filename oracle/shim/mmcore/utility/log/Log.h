// Minimal stand-in for MegaMol's logger (core/include/mmcore/utility/log/Log.h), oracle build only.
// Messages are printf-formatted; errors go to stderr, info is dropped unless P2V_ORACLE_VERBOSE is set.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <cstdlib>

namespace megamol::core::utility::log {

class Log {
public:
    static Log DefaultLog;

    void WriteInfo(const char* fmt, ...) {
        if (std::getenv("P2V_ORACLE_VERBOSE") == nullptr)
            return;
        va_list ap;
        va_start(ap, fmt);
        std::vfprintf(stderr, fmt, ap);
        va_end(ap);
        std::fputc('\n', stderr);
    }

    void WriteWarn(const char* fmt, ...) {
        va_list ap;
        va_start(ap, fmt);
        std::vfprintf(stderr, fmt, ap);
        va_end(ap);
        std::fputc('\n', stderr);
    }

    void WriteError(const char* fmt, ...) {
        va_list ap;
        va_start(ap, fmt);
        std::vfprintf(stderr, fmt, ap);
        va_end(ap);
        std::fputc('\n', stderr);
    }
};

inline Log Log::DefaultLog;

} // namespace megamol::core::utility::log
