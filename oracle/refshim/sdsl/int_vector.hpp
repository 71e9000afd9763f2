// Test-infrastructure shim (oracle build only): stands in for the sdsl-lite
// library (absent here).  int_vector<0> stores full 64-bit words; the reference
// only ever stores values that fit the declared width (MinimizerSeeder.cpp:318,
// 452), so the stored values are identical to the bit-packed original.
#pragma once
#include <vector>
#include <cstdint>
#include <cstddef>
namespace sdsl {
template <int W>
class int_vector
{
public:
	using value_type = uint64_t;
	using iterator = std::vector<uint64_t>::iterator;
	using const_iterator = std::vector<uint64_t>::const_iterator;
	int_vector() : w(64) {}
	void width(int nw) { w = nw; }
	int width() const { return w; }
	void resize(size_t n) { data.resize(n, 0); }
	size_t size() const { return data.size(); }
	uint64_t& operator[](size_t i) { return data[i]; }
	uint64_t operator[](size_t i) const { return data[i]; }
	iterator begin() { return data.begin(); }
	iterator end() { return data.end(); }
	const_iterator begin() const { return data.begin(); }
	const_iterator end() const { return data.end(); }
private:
	std::vector<uint64_t> data;
	int w;
};
namespace util {
template <typename V> void set_to_value(V& v, uint64_t value) { for (auto& x : v) x = value; }
}
}
