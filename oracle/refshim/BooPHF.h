// Test-infrastructure shim (oracle build only): stands in for the un-vendored
// BBHash minimal perfect hash.  lookup() returns the rank of the key among the
// sorted distinct keys, or ULLONG_MAX for keys outside the set.  Seeding results
// do not depend on which dense id a key receives (hits are verified through
// kmerCheck, MinimizerSeeder.cpp:531) except through initMaxCount's exclusion
// of the last id (MinimizerSeeder.cpp:564); with this shim the last id is the
// numerically largest k-mer.
#pragma once
#include <vector>
#include <algorithm>
#include <unordered_map>
#include <cstdint>
#include <climits>
namespace boomphf {
template <typename T> struct SingleHashFunctor {};
template <typename Key, typename Hasher>
class mphf
{
public:
	template <typename Range>
	mphf(size_t n, const Range& keys, int threads, double gamma, bool writeEach, bool progress)
	{
		std::vector<Key> sorted(keys.begin(), keys.end());
		std::sort(sorted.begin(), sorted.end());
		sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
		index.reserve(sorted.size());
		for (size_t i = 0; i < sorted.size(); i++) index.emplace(sorted[i], i);
		(void)n; (void)threads; (void)gamma; (void)writeEach; (void)progress;
	}
	uint64_t lookup(const Key& key) const
	{
		auto found = index.find(key);
		if (found == index.end()) return ULLONG_MAX;
		return found->second;
	}
	uint64_t nbKeys() const { return index.size(); }
private:
	std::unordered_map<Key, uint64_t> index;
};
}
