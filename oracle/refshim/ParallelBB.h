// Test-infrastructure shim (oracle build only); declarations live in BooPHF.h.
#pragma once
#include "BooPHF.h"
