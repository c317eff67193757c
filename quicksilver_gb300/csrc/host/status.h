// Thread-local error text behind qsg_last_error() and the helpers every
// entry point uses to turn a failure into a status code.
#pragma once

#include <cstdarg>
#include <string>

#include "qsg.h"

namespace qsg {

// Record `fmt` as the calling thread's last error and return `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();
const std::string& last_error();

}  // namespace qsg

// Wrap an entry point body: exceptions never cross the C ABI.
#define QSG_API_BEGIN try {
#define QSG_API_END                                                            \
    }                                                                          \
    catch (const std::bad_alloc&) {                                            \
        return qsg::fail(QSG_ERR_CAPACITY, "host allocation failed");          \
    }                                                                          \
    catch (const std::exception& e) {                                          \
        return qsg::fail(QSG_ERR_INVALID, "%s", e.what());                     \
    }                                                                          \
    catch (...) {                                                              \
        return qsg::fail(QSG_ERR_INVALID, "unknown exception");                \
    }
