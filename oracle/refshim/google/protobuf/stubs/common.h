// Test-infrastructure shim (oracle build only): minimal protobuf declarations
// so the reference's stream.hpp compiles.  Protobuf streams are never used on
// the GFA path the oracle exercises; every method reports end-of-input.
#pragma once
#include <cstdint>
#include <string>
#include <istream>
#include <ostream>
namespace google { namespace protobuf {
typedef uint64_t uint64;
typedef uint32_t uint32;
namespace io {
class ZeroCopyInputStream { public: virtual ~ZeroCopyInputStream() {} };
class ZeroCopyOutputStream { public: virtual ~ZeroCopyOutputStream() {} };
class IstreamInputStream : public ZeroCopyInputStream { public: explicit IstreamInputStream(std::istream*) {} };
class OstreamOutputStream : public ZeroCopyOutputStream { public: explicit OstreamOutputStream(std::ostream*) {} };
class GzipInputStream : public ZeroCopyInputStream { public: explicit GzipInputStream(ZeroCopyInputStream*) {} };
class GzipOutputStream : public ZeroCopyOutputStream { public: explicit GzipOutputStream(ZeroCopyOutputStream*) {} void Close() {} };
class CodedInputStream {
public:
	explicit CodedInputStream(ZeroCopyInputStream*) {}
	bool ReadVarint64(uint64* v) { *v = 0; return false; }
	bool ReadVarint32(uint32* v) { *v = 0; return false; }
	bool ReadString(std::string*, int) { return false; }
};
class CodedOutputStream {
public:
	explicit CodedOutputStream(ZeroCopyOutputStream*) {}
	void WriteVarint64(uint64) {}
	void WriteVarint32(uint32) {}
	void WriteString(const std::string&) {}
	void WriteRaw(const void*, int) {}
};
} } }
