// Test-infrastructure shim (oracle build only): stands in for the un-vendored
// zstr submodule.  The oracle driver reads plain (uncompressed) FASTA itself,
// so zstr::ifstream is a plain std::ifstream here.
#pragma once
#include <fstream>
namespace zstr { using ifstream = std::ifstream; }
