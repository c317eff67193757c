#include "status.h"

#include <cstdio>
#include <cstring>

namespace qsg {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

void clear_error() { g_last_error.clear(); }

const std::string& last_error() { return g_last_error; }

}  // namespace qsg

extern "C" int qsg_abi_version(void) { return QSG_ABI_VERSION; }

extern "C" int qsg_last_error(char* buf, size_t len)
{
    if (!buf || len == 0) return QSG_ERR_INVALID;
    const std::string& e = qsg::last_error();
    size_t n = e.size() < len - 1 ? e.size() : len - 1;
    memcpy(buf, e.data(), n);
    buf[n] = '\0';
    return QSG_OK;
}
