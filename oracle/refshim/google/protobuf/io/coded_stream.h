// Test-infrastructure shim (oracle build only); declarations live in stubs/common.h.
#pragma once
#include "google/protobuf/stubs/common.h"
