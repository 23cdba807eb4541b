// hss_api_status.h - status codes and limits shared by the host sources.
#pragma once
#include "../../include/hss.h"

namespace hss {
constexpr uint64_t kMaxLimit = HSS_MAX_LIMIT;
}
