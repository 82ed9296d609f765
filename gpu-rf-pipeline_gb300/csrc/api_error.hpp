// Sets the message rfx_last_error() returns on this thread and passes `status` through; for
// C ABI entry points defined outside rfx_api.cu.
#pragma once

namespace rfx {

int set_last_error(int status, const char* message);

}  // namespace rfx
