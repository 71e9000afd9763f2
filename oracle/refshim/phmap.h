// Test-infrastructure shim (oracle build only): stands in for the un-vendored
// parallel-hashmap submodule that the reference source includes as <phmap.h>.
//
// phmap::flat_hash_map is replaced by an insertion-ordered hash map.  The
// reference iterates these maps when it seeds the component priority queue
// from the previous band (GraphAlignerBitvectorBanded.h:313) and when it
// groups seeds (GraphAligner.h:280), so the iteration order is part of the
// observable behaviour in cyclic-component tie cases.  Insertion order is the
// documented, deterministic order this oracle pins; the GPU path reproduces
// it (a slice's band is kept in first-pop order).  Element references stay
// valid across insertions (std::deque storage), which the reference relies
// on (GraphAlignerBitvectorBanded.h:393).
#pragma once
#include <cstddef>
#include <deque>
#include <unordered_map>
#include <utility>
#include <stdexcept>
#include <functional>

namespace phmap
{

template <typename K, typename V, typename Hash = std::hash<K>, typename Eq = std::equal_to<K>, typename Alloc = void>
class flat_hash_map
{
public:
	using key_type = K;
	using mapped_type = V;
	using value_type = std::pair<K, V>;
	using storage = std::deque<value_type>;
	using iterator = typename storage::iterator;
	using const_iterator = typename storage::const_iterator;

	flat_hash_map() = default;
	flat_hash_map(const flat_hash_map& other) : items(other.items), index()
	{
		rebuild();
	}
	flat_hash_map(flat_hash_map&& other) = default;
	flat_hash_map& operator=(const flat_hash_map& other)
	{
		items = other.items;
		rebuild();
		return *this;
	}
	flat_hash_map& operator=(flat_hash_map&& other) = default;

	V& operator[](const K& key)
	{
		auto found = index.find(key);
		if (found != index.end()) return items[found->second].second;
		index.emplace(key, items.size());
		items.emplace_back(key, V());
		return items.back().second;
	}
	V& at(const K& key)
	{
		auto found = index.find(key);
		if (found == index.end()) throw std::out_of_range("phmap shim: key not found");
		return items[found->second].second;
	}
	const V& at(const K& key) const
	{
		auto found = index.find(key);
		if (found == index.end()) throw std::out_of_range("phmap shim: key not found");
		return items[found->second].second;
	}
	iterator find(const K& key)
	{
		auto found = index.find(key);
		if (found == index.end()) return items.end();
		return items.begin() + found->second;
	}
	const_iterator find(const K& key) const
	{
		auto found = index.find(key);
		if (found == index.end()) return items.end();
		return items.begin() + found->second;
	}
	size_t count(const K& key) const { return index.count(key); }
	size_t size() const { return items.size(); }
	bool empty() const { return items.empty(); }
	void reserve(size_t n) { index.reserve(n); }
	void resize(size_t n) { index.reserve(n); }
	void clear() { items.clear(); index.clear(); }
	iterator begin() { return items.begin(); }
	iterator end() { return items.end(); }
	const_iterator begin() const { return items.begin(); }
	const_iterator end() const { return items.end(); }
	std::pair<iterator, bool> insert(const value_type& v)
	{
		auto found = index.find(v.first);
		if (found != index.end()) return std::make_pair(items.begin() + found->second, false);
		index.emplace(v.first, items.size());
		items.push_back(v);
		return std::make_pair(items.end() - 1, true);
	}
	template <typename... Args>
	std::pair<iterator, bool> emplace(const K& key, Args&&... args)
	{
		auto found = index.find(key);
		if (found != index.end()) return std::make_pair(items.begin() + found->second, false);
		index.emplace(key, items.size());
		items.emplace_back(std::piecewise_construct, std::forward_as_tuple(key), std::forward_as_tuple(std::forward<Args>(args)...));
		return std::make_pair(items.end() - 1, true);
	}
private:
	void rebuild()
	{
		index.clear();
		index.reserve(items.size());
		for (size_t i = 0; i < items.size(); i++) index.emplace(items[i].first, i);
	}
	storage items;
	std::unordered_map<K, size_t, Hash, Eq> index;
};

template <typename K, typename Hash = std::hash<K>, typename Eq = std::equal_to<K>, typename Alloc = void>
class flat_hash_set
{
public:
	using storage = std::deque<K>;
	using iterator = typename storage::const_iterator;
	using const_iterator = typename storage::const_iterator;
	std::pair<iterator, bool> insert(const K& key)
	{
		auto found = index.find(key);
		if (found != index.end()) return std::make_pair(items.cbegin() + found->second, false);
		index.emplace(key, items.size());
		items.push_back(key);
		return std::make_pair(items.cend() - 1, true);
	}
	size_t count(const K& key) const { return index.count(key); }
	size_t size() const { return items.size(); }
	const_iterator begin() const { return items.begin(); }
	const_iterator end() const { return items.end(); }
	void clear() { items.clear(); index.clear(); }
private:
	storage items;
	std::unordered_map<K, size_t, Hash, Eq> index;
};

}
