// engine.h -- engine entry points used by other translation units.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/hbx.h"

namespace hbx {

// Runs a session (batched or plain) on its context's stream and copies its
// pairs, exactly sized, into host vectors.
void run_to_host(hbx_session* s, hbx_mode mode, std::vector<uint32_t>* l, std::vector<uint32_t>* r);

}  // namespace hbx
