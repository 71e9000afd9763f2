// Test-infrastructure shim (oracle build only); see int_vector.hpp.
#pragma once
#include "int_vector.hpp"
