// Test-infrastructure shim (oracle build only): stands in for the un-vendored
// moodycamel concurrentqueue submodule with a mutex-protected FIFO offering the
// calls the reference makes (enqueue / try_dequeue / producer tokens).
#pragma once
#include <deque>
#include <mutex>
namespace moodycamel {
template <typename T>
class ConcurrentQueue
{
public:
	ConcurrentQueue() {}
	explicit ConcurrentQueue(size_t) {}
	ConcurrentQueue(ConcurrentQueue&& other) : items(std::move(other.items)) {}
	ConcurrentQueue& operator=(ConcurrentQueue&& other) { items = std::move(other.items); return *this; }
	bool enqueue(const T& item) { std::lock_guard<std::mutex> g { lock }; items.push_back(item); return true; }
	template <typename Token> bool enqueue(Token&, const T& item) { return enqueue(item); }
	bool try_dequeue(T& out) { std::lock_guard<std::mutex> g { lock }; if (items.empty()) return false; out = items.front(); items.pop_front(); return true; }
	size_t size_approx() const { return items.size(); }
private:
	std::deque<T> items;
	std::mutex lock;
};
struct ProducerToken { template <typename Q> explicit ProducerToken(Q&) {} };
}
