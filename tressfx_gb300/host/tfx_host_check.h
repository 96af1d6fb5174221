// Status check shared by the host classes: a failing C-ABI call becomes a TressFXError.
#pragma once
#include <string>

#include "tressfx/TressFXCommon.h"

namespace tfxhost {
inline void check(int status, const char* what) {
    if (status != TFX_OK) throw TressFXError(status, std::string(what) + ": " + tfx_last_error());
}
}  // namespace tfxhost
