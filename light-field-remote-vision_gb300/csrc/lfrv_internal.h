// lfrv_internal.h -- shared host-side helpers of liblfrv (error reporting, status plumbing).
#pragma once

#include "lfrv.h"

#include <cstdarg>
#include <cstdio>
#include <string>

namespace lfrv {

// Records a message for lfrv_last_error() (thread-local) and returns the status unchanged.
int fail(int status, const char *fmt, ...);

// Exception used inside the library; every extern "C" entry point converts it into a status code.
struct Error {
    int status;
    std::string msg;
};

[[noreturn]] void raise(int status, const char *fmt, ...);

}  // namespace lfrv

// Wraps the body of an extern "C" entry point.
#define LFRV_API_BEGIN try {
#define LFRV_API_END                                                  \
    }                                                                 \
    catch (const lfrv::Error &e) {                                    \
        return lfrv::fail(e.status, "%s", e.msg.c_str());             \
    }                                                                 \
    catch (const std::bad_alloc &) {                                  \
        return lfrv::fail(LFRV_E_NOMEM, "host allocation failed");    \
    }                                                                 \
    catch (...) {                                                     \
        return lfrv::fail(LFRV_E_ARG, "unexpected C++ exception");    \
    }                                                                 \
    return LFRV_OK;
