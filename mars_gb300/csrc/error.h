// Error type shared by host and device translation units.
#pragma once

#include <stdexcept>
#include <string>

namespace mgpu {

// Error carrying a C-ABI status code; converted to a status at the ABI edge.
struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string &msg) : std::runtime_error(msg), status(st) {}
};

// Records the message returned by mars_gpu_last_error() on this thread.
void set_last_error(const std::string &msg);

inline void verify(bool ok, const char *msg, int status = 1)
{
    if (!ok) {
        throw Error(status, msg);
    }
}

}  // namespace mgpu
