// include/timer.hpp of the GB300 drop-in: Time, ElapsedTime (core.hpp) and the
// device-synchronised PlatformTime / GlobalPlatformTime (platform.hpp), under the
// header name the reference's drivers include.
#pragma once

#include "core.hpp"
#include "platform.hpp"
