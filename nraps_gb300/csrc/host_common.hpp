/* host_common.hpp — error text shared by the host-side entry points. */
#ifndef NRAPS_HOST_COMMON_HPP
#define NRAPS_HOST_COMMON_HPP
#include <string>

struct nraps_ctx;

namespace nraps_host {
/* Message of the last failure of a call made without a context, per thread. */
void set_error(const std::string& msg);
const char* last_error();
/* Records msg as the context's last error (nraps_last_error(ctx)). */
void set_ctx_error(nraps_ctx* ctx, const std::string& msg);
}  // namespace nraps_host
#endif
