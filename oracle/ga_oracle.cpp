// ORACLE — test infrastructure, not product code.
//
// A CPU restatement of GraphAligner's seed-extension path
// (GraphAlignerBitvectorBanded::getReverseTraceFromSeed and everything it
// calls), used only by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg to check and time the GPU kernels.  Each function cites the
// reference file:line it restates.  Its outputs are pinned against the
// reference itself (oracle/_ref/ga_ref built from the reference's own source;
// golden vectors in tests/golden/).
//
// Exported C ABI (ctypes): ora_extend_batch() takes the same graph / request /
// result structs as the GPU entry point ga_extend_batch() in
// include/graphaligner_gb300.h, and runs extensions on `threads` host threads.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <cstring>
#include <functional>
#include <queue>
#include <stdexcept>
#include <thread>
#include <unordered_map>
#include <vector>
#include "../include/graphaligner_gb300.h"

namespace ora
{
using u64 = uint64_t;
using i32 = int32_t;
static constexpr u64 AllOnes = ~0ULL;
static constexpr u64 LastBit = 1ULL << 63;

struct AssertFail {};
struct CapacityFail {};
#define ORA_ASSERT(x) do { if (!(x)) throw ::ora::AssertFail{}; } while (0)

static inline int popc(u64 x) { return __builtin_popcountll(x); }
// two's-complement int32 arithmetic without C++ overflow UB
static inline i32 add(i32 a, i32 b) { return (i32)((uint32_t)a + (uint32_t)b); }
static inline i32 sub(i32 a, i32 b) { return (i32)((uint32_t)a - (uint32_t)b); }
static inline i32 mul(i32 a, i32 b) { return (i32)((uint32_t)a * (uint32_t)b); }

// WordSlice (WordSlice.h:150-260): a 64-row column as VP/VN plus the last row's score.
struct WS
{
	u64 VP = 0;
	u64 VN = 0;
	i32 scoreEnd = 0;
	bool operator==(const WS& o) const { return VP == o.VP && VN == o.VN && scoreEnd == o.scoreEnd; }
};

static inline i32 getValue(const WS& w, int row)   // WordSlice.h:177-186
{
	u64 mask = 0;
	if (row < 63) mask = AllOnes << (row + 1);
	return sub(add(w.scoreEnd, popc(w.VN & mask)), popc(w.VP & mask));
}
static inline i32 scoreBeforeStart(const WS& w)    // WordSlice.h:244-247
{
	return add(sub(w.scoreEnd, popc(w.VP)), popc(w.VN));
}
static inline i32 getXScore(const WS& w, i32 seqOffset, int offset, i32 cost)  // WordSlice.h:239-242
{
	return sub(mul(add(add(seqOffset, offset), 1), 100), mul(getValue(w, offset), cost));
}

// WordSlice::maxXScoreLocalMinima (WordSlice.h:313-347)
static i32 maxXScore(const WS& w, i32 seqOffset, i32 cost, int cells = 64, u64 extraMask = AllOnes)
{
	i32 sbs = scoreBeforeStart(w);
	u64 pcm = ~w.VP;
	u64 plm = w.VP & (pcm - w.VP);
	plm >>= 1;
	plm |= LastBit & (pcm | ~(pcm - w.VP)) & ~w.VP;
	i32 result = INT32_MIN;
	plm &= extraMask;
	plm |= 1;
	if (cells < 64)
	{
		plm |= 1ULL << (cells - 1);
		plm &= ~(AllOnes << cells);
	}
	else
	{
		plm |= 1ULL << 63;
	}
	i32 zeroScore = sub(mul(seqOffset, 100), mul(sbs, cost));
	while (plm != 0)
	{
		u64 m = plm ^ (plm - 1);
		i32 cellsHere = popc(m);
		i32 scoreHere = popc(w.VP & m) - popc(w.VN & m);
		result = std::max(result, sub(mul(cellsHere, 100), mul(scoreHere, cost)));
		plm &= ~m;
	}
	return add(result, zeroScore);
}

// WordSlice::differenceMasksBitTwiddle (WordSlice.h:566-664)
static std::pair<u64, u64> differenceMasks(u64 leftVP, u64 leftVN, u64 rightVP, u64 rightVN, int scoreDifference)
{
	u64 leftSmaller = 0;
	u64 rightSmaller = 0;
	u64 VPcommon = ~(leftVP & rightVP);
	u64 VNcommon = ~(leftVN & rightVN);
	leftVP &= VPcommon;
	leftVN &= VNcommon;
	rightVP &= VPcommon;
	rightVN &= VNcommon;
	u64 twosmaller = leftVN & rightVP;
	u64 onesmaller = (rightVP & ~leftVN) | (leftVN & ~rightVP);
	u64 onebigger = (leftVP & ~rightVN) | (rightVN & ~leftVP);
	u64 twobigger = rightVN & leftVP;
	onebigger |= twobigger;
	onesmaller |= twosmaller;
	if (scoreDifference > 0)
	{
		for (int i = 1; i < scoreDifference; i++)
		{
			u64 ls = onebigger & ~(onebigger - 1);
			onebigger ^= (~twobigger & ls);
			twobigger &= ~ls;
			if (onebigger == 0) return { AllOnes, 0 };
		}
		u64 ls = onebigger & ~(onebigger - 1);
		leftSmaller |= ls - 1;
		onebigger ^= (~twobigger & ls);
		twobigger &= ~ls;
	}
	else if (scoreDifference < 0)
	{
		for (int i = 1; i < -scoreDifference; i++)
		{
			u64 ls = onesmaller & ~(onesmaller - 1);
			onesmaller ^= (~twosmaller & ls);
			twosmaller &= ~ls;
			if (onesmaller == 0) return { 0, AllOnes };
		}
		u64 ls = onesmaller & ~(onesmaller - 1);
		rightSmaller |= ls - 1;
		onesmaller ^= (~twosmaller & ls);
		twosmaller &= ~ls;
	}
	for (int i = 0; i < 64; i++)
	{
		if (onesmaller == 0)
		{
			if (onebigger == 0) break;
			u64 ls = onebigger & ~(onebigger - 1);
			rightSmaller |= -ls;
			break;
		}
		if (onebigger == 0)
		{
			u64 ls = onesmaller & ~(onesmaller - 1);
			leftSmaller |= -ls;
			break;
		}
		u64 lsB = onebigger & ~(onebigger - 1);
		u64 lsS = onesmaller & ~(onesmaller - 1);
		if (lsB > lsS) leftSmaller |= lsB - lsS;
		else rightSmaller |= lsS - lsB;
		onebigger ^= (~twobigger & lsB);
		twobigger &= ~lsB;
		onesmaller ^= (~twosmaller & lsS);
		twosmaller &= ~lsS;
	}
	return { leftSmaller, rightSmaller };
}

// WordSlice::mergeTwoSlices (WordSlice.h:502-541)
static WS merge(WS left, WS right)
{
	if (scoreBeforeStart(left) > scoreBeforeStart(right)) std::swap(left, right);
	auto masks = differenceMasks(left.VP, left.VN, right.VP, right.VN, sub(scoreBeforeStart(right), scoreBeforeStart(left)));
	u64 leftSmaller = masks.first;
	u64 rightSmaller = masks.second;
	u64 mask = (rightSmaller | ((leftSmaller | rightSmaller) - (rightSmaller << 1))) & ~leftSmaller;
	u64 leftReduction = leftSmaller & (rightSmaller << 1);
	u64 rightReduction = rightSmaller & (leftSmaller << 1);
	if ((rightSmaller & 1) && scoreBeforeStart(left) < scoreBeforeStart(right)) rightReduction |= 1;
	left.VN &= ~leftReduction;
	right.VN &= ~rightReduction;
	WS result;
	result.VN = (left.VN & ~mask) | (right.VN & mask);
	result.VP = (left.VP & ~mask) | (right.VP & mask);
	result.scoreEnd = std::min(left.scoreEnd, right.scoreEnd);
	return result;
}

// WordSlice::changedMinScoreLocalMinima (WordSlice.h:438-472)
static i32 changedMinScore(const WS& w, const WS& old)
{
	i32 sbs = scoreBeforeStart(w);
	i32 osbs = scoreBeforeStart(old);
	u64 plm = w.VP & (w.VN - w.VP);
	plm >>= 1;
	plm |= LastBit & (w.VN | ~(w.VN - w.VP)) & ~w.VP;
	if (add(w.scoreEnd, popc(w.VN)) >= sub(old.scoreEnd, popc(old.VP)))
	{
		u64 smaller = differenceMasks(w.VP, w.VN, old.VP, old.VN, sub(osbs, sbs)).first;
		if (smaller != AllOnes)
		{
			plm |= (~smaller) >> 1;
			plm |= (~smaller) << 1;
			plm |= 1;
			plm |= LastBit;
			plm &= smaller;
		}
	}
	i32 result = (sbs < osbs) ? sbs : INT32_MAX;
	while (plm != 0)
	{
		u64 m = plm ^ (plm - 1);
		i32 sh = sub(add(sbs, popc(w.VP & m)), popc(w.VN & m));
		result = std::min(result, sh);
		plm &= ~m;
	}
	return result;
}

// GraphAlignerBitvectorCommon::getNextSlice (GraphAlignerBitvectorCommon.h:242-262), Myers 1999
static inline WS nextSlice(u64 Eq, WS s, u64 hinP, u64 hinN, u64& Ph, u64& Mh)
{
	u64 Xv = Eq | s.VN;
	Eq |= hinN;
	u64 Xh = (((Eq & s.VP) + s.VP) ^ s.VP) | Eq;
	Ph = s.VN | ~(Xh | s.VP);
	Mh = s.VP & Xh;
	u64 tempMh = (Mh << 1) | hinN;
	u64 outN = Mh >> 63;
	u64 tempPh = (Ph << 1) | hinP;
	s.VP = tempMh | ~(Xv | tempPh);
	u64 outP = Ph >> 63;
	s.VN = tempPh & Xv;
	s.scoreEnd = sub(s.scoreEnd, (i32)outN);
	s.scoreEnd = add(s.scoreEnd, (i32)outP);
	return s;
}

static inline WS sourceSlice(i32 previousScore)     // getSourceSliceFromScore (Common.h:1056-1060)
{
	WS r;
	r.VP = AllOnes;
	r.VN = 0;
	r.scoreEnd = add(previousScore, 64);
	return r;
}

// IUPAC matching, GraphAlignerCommon::characterMatch / ambiguousMatch (GraphAlignerCommon.h:176-279)
static int iupacMask(char c)   // bit0 A, bit1 C, bit2 G, bit3 T; -1 = invalid (reference asserts)
{
	switch (c)
	{
		case 'A': case 'a': return 1;
		case 'C': case 'c': return 2;
		case 'G': case 'g': return 4;
		case 'T': case 't': case 'U': case 'u': return 8;
		case 'R': case 'r': return 1 | 4;
		case 'Y': case 'y': return 2 | 8;
		case 'K': case 'k': return 4 | 8;
		case 'M': case 'm': return 2 | 1;
		case 'S': case 's': return 2 | 4;
		case 'W': case 'w': return 1 | 8;
		case 'B': case 'b': return 2 | 4 | 8;
		case 'D': case 'd': return 1 | 4 | 8;
		case 'H': case 'h': return 1 | 2 | 8;
		case 'V': case 'v': return 1 | 2 | 4;
		case 'N': case 'n': return 15;
		case '-': return 0;
	}
	return -1;
}
static bool characterMatch(char seq, char graph)
{
	if (seq == graph) return true;
	int a = iupacMask(seq);
	int b = iupacMask(graph);
	ORA_ASSERT(a >= 0 && b >= 0);
	return (a & b) != 0;
}

// 64-row match masks (getEqVector, Common.h:279-318): masks[0..3] = A, C, G, T
struct EqV { u64 m[4]; };
static EqV getEq(const char* seq, size_t len, size_t j)
{
	EqV r { {0, 0, 0, 0} };
	for (int i = 0; i < 64 && j + i < len; i++)
	{
		int mask = iupacMask(seq[j + i]);
		// getEqVector (Common.h:307-315): a non-sequence byte asserts in ambiguousMatch;
		// a gap only fails the full-window check
		ORA_ASSERT(mask >= 0);
		ORA_ASSERT(mask != 0 || j + 64 > len);
		for (int c = 0; c < 4; c++) if (mask & (1 << c)) r.m[c] |= 1ULL << i;
	}
	return r;
}

struct Graph
{
	const ga_graph_desc* d;
	uint32_t len(uint32_t n) const { return d->node_length[n]; }
	// Eq mask for a node column (EqVector::getEqI, Common.h:46-55,113-117)
	u64 eqAt(const EqV& e, uint32_t n, uint32_t pos) const
	{
		if (n < d->first_ambiguous)
		{
			u64 chunk = d->seq2bit[(size_t)n * 2 + pos / 32];
			return e.m[(chunk >> ((pos % 32) * 2)) & 3];
		}
		const u64* a = d->seq_ambiguous + (size_t)(n - d->first_ambiguous) * 4;
		u64 r = 0;
		for (int c = 0; c < 4; c++) if ((a[c] >> pos) & 1) r |= e.m[c];
		return r;
	}
	// AlignmentGraph::NodeSequences (AlignmentGraph.cpp:734-773)
	char charAt(uint32_t n, uint32_t pos) const
	{
		if (n < d->first_ambiguous)
		{
			u64 chunk = d->seq2bit[(size_t)n * 2 + pos / 32];
			return "ACGT"[(chunk >> ((pos % 32) * 2)) & 3];
		}
		const u64* a = d->seq_ambiguous + (size_t)(n - d->first_ambiguous) * 4;
		int m = 0;
		for (int c = 0; c < 4; c++) if ((a[c] >> pos) & 1) m |= 1 << c;
		static const char table[16] = { '?', 'A', 'C', 'M', 'G', 'R', 'S', 'V', 'T', 'W', 'Y', 'H', 'K', 'D', 'B', 'N' };
		return table[m];
	}
	const uint32_t* inBegin(uint32_t n) const { return d->in_neighbors + d->in_offsets[n]; }
	const uint32_t* inEnd(uint32_t n) const { return d->in_neighbors + d->in_offsets[n + 1]; }
	uint32_t inCount(uint32_t n) const { return d->in_offsets[n + 1] - d->in_offsets[n]; }
	const uint32_t* outBegin(uint32_t n) const { return d->out_neighbors + d->out_offsets[n]; }
	const uint32_t* outEnd(uint32_t n) const { return d->out_neighbors + d->out_offsets[n + 1]; }
};

// NodeSliceMapItemStruct (NodeSlice.h:15-47), one 64-bp node
struct Item
{
	WS startSlice;
	WS endSlice;
	bool exists = false;
	u64 HP = 0;
	u64 HN = 0;
	i32 minScore = 0;
	// multiseed DP only: DPSlice::seedstartNodes and DPSlice::nodeMaxExactEndposScore
	// (Common.h:184-185) kept with the node's band entry
	bool seedStart = false;
	i32 nodeMax = 0;
};

// One band: node -> item in first-insertion order (see refshim/phmap.h)
struct Band
{
	std::vector<uint32_t> nodes;
	std::vector<Item> items;
	std::unordered_map<uint32_t, uint32_t> index;
	bool has(uint32_t n) const { return index.count(n) != 0; }
	Item& at(uint32_t n) { auto f = index.find(n); ORA_ASSERT(f != index.end()); return items[f->second]; }
	const Item& at(uint32_t n) const { auto f = index.find(n); ORA_ASSERT(f != index.end()); return items[f->second]; }
	Item& add(uint32_t n)
	{
		auto f = index.find(n);
		if (f != index.end()) return items[f->second];
		index.emplace(n, (uint32_t)items.size());
		nodes.push_back(n);
		items.emplace_back();
		return items.back();
	}
	size_t size() const { return items.size(); }
};

// DPSlice (Common.h:137-213)
struct Slice
{
	int64_t j = 0;
	i32 minScore = INT32_MAX;
	size_t minScoreNode = SIZE_MAX;
	size_t minScoreNodeOffset = SIZE_MAX;
	i32 maxExactEndposScore = INT32_MIN;
	size_t maxExactEndposNode = SIZE_MAX;
	size_t cellsProcessed = 0;
	size_t bandwidth = 0;
	bool scoresNotValid = false;
	Band scores;
};

// EdgeWithPriority (GraphAlignerCommon.h:32-51), restricted to the fields the path uses
struct Edge
{
	uint32_t target;
	WS incoming;
	bool skipFirst;
	bool force = false;     // EdgeWithPriority::forceCalculation (a seed start)
};

// ComponentPriorityQueue (ComponentPriorityQueue.h:8-156): a std::priority_queue
// min-heap on (component, score) plus per-node pending incoming edges.
struct ComponentQueue
{
	struct P
	{
		size_t component;
		int score;
		size_t index;
		bool operator>(const P& o) const { return component > o.component || (component == o.component && score > o.score); }
	};
	std::priority_queue<P, std::vector<P>, std::greater<P>> heap;
	std::unordered_map<uint32_t, std::vector<Edge>> extras;
	void insert(size_t component, int score, const Edge& e)
	{
		auto& ex = extras[e.target];
		if (ex.empty()) heap.push(P { component, score, e.target });
		ex.push_back(e);
	}
	size_t size() const { return heap.size(); }
	uint32_t topIndex() const { return (uint32_t)heap.top().index; }
	void pop()
	{
		extras[(uint32_t)heap.top().index].clear();
		heap.pop();
	}
	void clear()
	{
		while (!heap.empty()) pop();
		extras.clear();
	}
};

struct NodeCalc
{
	i32 minScore;
	size_t minScoreNode;
	size_t minScoreNodeOffset;
	size_t maxExactEndposNode;
	i32 maxExactEndposScore;
	size_t cellsProcessed;
};

struct Params
{
	size_t bandwidth;
	i32 xdrop;
	size_t maxCells;
	i32 cost;
	double multimapScoreFraction = 0.9;
};

static inline bool isFake(const WS& w) { return w.scoreEnd == INT32_MAX; }
static const WS FakeSlice { 0, 0, INT32_MAX };

// calculateNodeInner (GraphAlignerBitvectorCommon.h:1113-1478).  `extra` is the extraSlice:
// the single-seed path passes the fake slice (scoreEnd INT32_MAX) everywhere; the multiseed
// DP passes the seed-start slice (getSeedSlice) for a node that is a seed start in this slice.
// AllowEarlyLeave = true is the fill (calculateNodeClipPrecise, :1104-1111);
// false is recalcNodeWordslice (:1078-1102), which records every column.
template <bool AllowEarlyLeave>
static NodeCalc calcNode(const Graph& g, const Params& p, uint32_t i, Item& slice, const EqV& eqv, const Item& previousSlice,
	const std::vector<Edge>& incoming, const std::vector<char>* previousBandHas, i32 seqOffset,
	std::vector<WS>* columns, uint64_t& columnSteps, const WS& extra)
{
	const bool hasExtra = !isFake(extra);
	bool forceCalculation = false;
	ORA_ASSERT(incoming.size() > 0);
	WS ws;
	bool hasWs = false;
	NodeCalc result;
	result.minScore = INT32_MAX;
	result.minScoreNode = SIZE_MAX;
	result.minScoreNodeOffset = SIZE_MAX;
	result.maxExactEndposScore = INT32_MIN;
	result.maxExactEndposNode = SIZE_MAX;
	result.cellsProcessed = 0;
	uint32_t nodeLength = g.len(i);
	u64 Eq = g.eqAt(eqv, i, 0);
	bool hasSkipless = false;
	for (const auto& inc : incoming)
	{
		result.cellsProcessed++;
		if (inc.force) forceCalculation = true;
		if (inc.skipFirst)
		{
			ws = hasWs ? merge(ws, inc.incoming) : inc.incoming;
			hasWs = true;
			continue;
		}
		hasSkipless = true;
		u64 hinP, hinN;
		i32 compareHin = INT32_MAX;
		if (previousSlice.exists) compareHin = previousSlice.startSlice.scoreEnd;
		if (hasExtra) compareHin = std::min(compareHin, scoreBeforeStart(extra));
		i32 incBefore = scoreBeforeStart(inc.incoming);
		if (compareHin < incBefore) { hinP = 0; hinN = 1; }
		else if (compareHin > incBefore) { hinP = 1; hinN = 0; }
		else { hinP = 0; hinN = 0; }
		u64 Ph, Mh;
		WS newWs = nextSlice(Eq, inc.incoming, hinP, hinN, Ph, Mh);
		columnSteps++;
		if (!previousSlice.exists || scoreBeforeStart(newWs) < previousSlice.startSlice.scoreEnd)
		{
			newWs.VP &= AllOnes ^ 1;
			newWs.VN |= 1;
		}
		ws = hasWs ? merge(ws, newWs) : newWs;
		hasWs = true;
	}
	ORA_ASSERT(hasWs);
	result.minScore = ws.scoreEnd;
	result.minScoreNode = i;
	result.minScoreNodeOffset = 0;
	if (hasExtra) ws = merge(ws, extra);
	result.maxExactEndposScore = maxXScore(ws, seqOffset, p.cost);
	result.maxExactEndposNode = i;
	if (!forceCalculation && slice.exists)
	{
		uint32_t inCount = g.inCount(i);
		bool singleInBand = false;
		// the fill checks the previous band; recalcNodeWordslice's check is constant false (Common.h:1088)
		if (hasSkipless && inCount == 1 && previousBandHas) singleInBand = (*previousBandHas)[*g.inBegin(i)] != 0;
		if (hasSkipless && inCount == 1 && singleInBand)
		{
			if (ws.scoreEnd > slice.startSlice.scoreEnd)
			{
				if (AllowEarlyLeave) return result;
			}
			else if (ws.scoreEnd < slice.startSlice.scoreEnd)
			{
			}
			else
			{
				u64 newBigger = (ws.VP & ~slice.startSlice.VP) | (slice.startSlice.VN & ~ws.VN);
				u64 oldBigger = (slice.startSlice.VP & ~ws.VP) | (ws.VN & ~slice.startSlice.VN);
				if (newBigger > oldBigger)
				{
				}
				else if (oldBigger > newBigger)
				{
					if (AllowEarlyLeave) return result;
				}
				else if (newBigger == 0 && oldBigger == 0)
				{
					if (AllowEarlyLeave) return result;
				}
				else
				{
					WS test = merge(ws, slice.startSlice);
					if (test == slice.startSlice)
					{
						if (AllowEarlyLeave) return result;
					}
					ws = test;
				}
			}
		}
		else
		{
			WS test = merge(ws, slice.startSlice);
			// reproduces the reference's comparison test.VP == slice.startSlice.VN (Common.h:1282)
			if (test.scoreEnd == slice.startSlice.scoreEnd && test.VP == slice.startSlice.VP && test.VP == slice.startSlice.VN)
			{
				if (AllowEarlyLeave) return result;
			}
			ws = test;
		}
	}
	if (previousSlice.exists)
	{
		if (scoreBeforeStart(ws) > previousSlice.startSlice.scoreEnd)
		{
			ws = merge(ws, sourceSlice(previousSlice.startSlice.scoreEnd));
		}
	}
	slice.HP = 0;
	slice.HN = 0;
	u64 forceMask = 0;
	u64 fixedHP = previousSlice.HP;
	u64 fixedHN = previousSlice.HN;
	if (previousSlice.exists)
	{
		i32 scoreBefore = scoreBeforeStart(ws);
		i32 scoreComparison = previousSlice.startSlice.scoreEnd;
		ORA_ASSERT(scoreBefore <= scoreComparison);
		if (hasExtra)
		{
			// Common.h:1314-1362: the row above follows the lower of the previous slice's
			// bottom row and the seed start's score before the slice
			const i32 extraBefore = scoreBeforeStart(extra);
			scoreBefore = std::min(scoreBefore, extraBefore);
			if (scoreBefore < scoreComparison) forceMask |= 1;
			i32 adjustScore = std::min(scoreBefore, scoreComparison);
			for (uint32_t fixoffset = 1; fixoffset < 64 && fixoffset < nodeLength; fixoffset++)
			{
				i32 newScoreComparison = scoreComparison + (i32)((fixedHP >> fixoffset) & 1) - (i32)((fixedHN >> fixoffset) & 1);
				if (scoreBefore < extraBefore) scoreBefore += 1;
				u64 mask = 1ULL << fixoffset;
				if (scoreBefore < newScoreComparison) forceMask |= mask;
				i32 newAdjustScore = std::min(newScoreComparison, scoreBefore);
				ORA_ASSERT(newAdjustScore >= adjustScore - 1 && newAdjustScore <= adjustScore + 1);
				if (newAdjustScore == adjustScore - 1)
				{
					fixedHN |= mask;
					fixedHP &= ~mask;
				}
				else if (newAdjustScore == adjustScore)
				{
					fixedHP &= ~mask;
					fixedHN &= ~mask;
				}
				else
				{
					fixedHP |= mask;
					fixedHN &= ~mask;
				}
				adjustScore = newAdjustScore;
				scoreComparison = newScoreComparison;
			}
		}
		else if (scoreBefore < scoreComparison)
		{
			forceMask |= 1;
			for (int fixoffset = 1; fixoffset < 64; fixoffset++)
			{
				i32 newScoreComparison = scoreComparison + (i32)((fixedHP >> fixoffset) & 1) - (i32)((fixedHN >> fixoffset) & 1);
				u64 mask = 1ULL << fixoffset;
				ORA_ASSERT(scoreBefore <= newScoreComparison);
				if (scoreBefore < newScoreComparison)
				{
					fixedHP |= mask;
					fixedHN &= ~mask;
					forceMask |= mask;
				}
				if (scoreBefore == newScoreComparison)
				{
					fixedHP &= ~mask;
					fixedHN &= ~mask;
				}
				scoreBefore++;
				scoreComparison = newScoreComparison;
				if (scoreBefore >= scoreComparison) break;
			}
		}
	}
	else
	{
		forceMask = AllOnes;
	}
	slice.startSlice = ws;
	if (!AllowEarlyLeave) columns->push_back(ws);
	slice.exists = true;
	u64 forceEq = AllOnes;
	if (!previousSlice.exists) forceEq ^= 1;
	uint32_t pos = 1;
	for (; pos < nodeLength; pos++)
	{
		Eq = g.eqAt(eqv, i, pos) & forceEq;
		u64 newHP, newHN;
		WS newWs = nextSlice(Eq, ws, (fixedHP >> pos) & 1, (fixedHN >> pos) & 1, newHP, newHN);
		columnSteps++;
		if ((forceMask >> pos) & 1)
		{
			newWs.VP &= AllOnes ^ 1;
			newWs.VN |= 1;
		}
		u64 hinP, hinN;
		if (hasExtra)
		{
			newWs = merge(newWs, extra);
			ORA_ASSERT(newWs.scoreEnd >= ws.scoreEnd - 1 && newWs.scoreEnd <= ws.scoreEnd + 1);
			hinP = newWs.scoreEnd == ws.scoreEnd + 1 ? 1 : 0;
			hinN = newWs.scoreEnd == ws.scoreEnd - 1 ? 1 : 0;
		}
		else
		{
			hinP = newHP >> 63;
			hinN = newHN >> 63;
		}
		ws = newWs;
		if (ws.scoreEnd < result.minScore)
		{
			result.minScore = ws.scoreEnd;
			result.minScoreNodeOffset = pos;
		}
		result.maxExactEndposScore = std::max(result.maxExactEndposScore, maxXScore(ws, seqOffset, p.cost, 64, newHN));
		if (!AllowEarlyLeave) columns->push_back(ws);
		slice.HP |= hinP << pos;
		slice.HN |= hinN << pos;
	}
	result.cellsProcessed = pos;
	slice.endSlice = ws;
	return result;
}

// Per-thread reusable buffers (AlignerGraphsizedState, GraphAlignerCommon.h:52-81)
struct State
{
	std::vector<char> previousBand;
	std::vector<char> currentBand;
	std::vector<char> hasSeedStart;
	ComponentQueue queue;
	explicit State(size_t n) : previousBand(n, 0), currentBand(n, 0), hasSeedStart(n, 0) {}
};

// The seeds one multiseed slice starts (seedHits[seedhitStart, seedhitEnd) of calculateSlice),
// with the seed-start slice of that slice (getSeedSlice); none for the single-seed path.
struct SliceSeeds
{
	const uint32_t* nodes = nullptr;
	size_t count = 0;
	WS slice { 0, 0, INT32_MAX };
	bool store = false;     // storeNodeExactEndposScores
};

// GraphAlignerBitvectorBanded::calculateSlice (GraphAlignerBitvectorBanded.h:255-511),
// component-queue branch; seeds (multiseed DP) as addSeedHitToScoresAndQueue (:228-253).
static NodeCalc calculateSlice(const Graph& g, const Params& p, const char* seq, size_t seqLen, size_t j,
	Band& currentSlice, const Band& previousSlice, State& st, i32 previousQuitScore, int bandwidth, i32 previousMinScore,
	uint64_t& columnSteps, const SliceSeeds& seeds = SliceSeeds())
{
	const bool multiseed = !isFake(seeds.slice);
	if (previousMinScore == INT32_MAX - bandwidth - 1)
	{
		ORA_ASSERT(multiseed);
		previousMinScore = scoreBeforeStart(seeds.slice);
		previousQuitScore = add(scoreBeforeStart(seeds.slice), bandwidth);
	}
	if (multiseed && previousMinScore > seeds.slice.scoreEnd)
	{
		previousMinScore = seeds.slice.scoreEnd;
		previousQuitScore = add(seeds.slice.scoreEnd, bandwidth);
	}
	NodeCalc result;
	result.minScore = INT32_MAX - bandwidth - 1;
	result.minScoreNode = SIZE_MAX;
	result.minScoreNodeOffset = SIZE_MAX;
	result.maxExactEndposNode = 0;
	result.maxExactEndposScore = INT32_MIN;
	result.cellsProcessed = 0;
	EqV eqv = getEq(seq, seqLen, j);
	ORA_ASSERT(previousSlice.size() > 0 || multiseed);
	for (size_t k = 0; k < previousSlice.size(); k++)
	{
		uint32_t node = previousSlice.nodes[k];
		const Item& item = previousSlice.items[k];
		if (j == 0)
		{
			ORA_ASSERT(item.minScore <= previousQuitScore);
		}
		else
		{
			if (item.minScore > previousQuitScore) continue;
			if (g.d->linearizable[node])
			{
				uint32_t nb = *g.inBegin(node);
				if (st.previousBand[nb] && previousSlice.at(nb).endSlice.scoreEnd < previousQuitScore && previousSlice.at(nb).minScore < previousQuitScore) continue;
			}
		}
		st.queue.insert(g.d->component[node], item.minScore, Edge { node, sourceSlice(item.startSlice.scoreEnd), true });
	}
	ORA_ASSERT(st.queue.size() > 0 || multiseed);
	if (multiseed && scoreBeforeStart(seeds.slice) < add(previousQuitScore, 64))
	{
		for (size_t k = 0; k < seeds.count; k++)
		{
			const uint32_t node = seeds.nodes[k];
			ORA_ASSERT(node < g.d->num_nodes);
			st.currentBand[node] = 1;
			Item& item = currentSlice.add(node);
			if (seeds.store) item.nodeMax = 0;
			item.minScore = seeds.slice.scoreEnd;
			item.startSlice = seeds.slice;
			item.endSlice = seeds.slice;
			item.exists = true;
			Edge e { node, seeds.slice, true };
			e.force = true;
			st.queue.insert(g.d->component[node], getValue(seeds.slice, 0), e);
			ORA_ASSERT(!st.hasSeedStart[node]);
			st.hasSeedStart[node] = 1;
			item.seedStart = true;
		}
	}
	i32 currentMinScoreAtEndRow = result.minScore;
	while (st.queue.size() > 0)
	{
		uint32_t i = st.queue.topIndex();
		if (!st.currentBand[i])
		{
			Item& added = currentSlice.add(i);
			added.minScore = INT32_MAX;
			added.startSlice = WS { 0, 0, INT32_MAX };
			added.endSlice = WS { 0, 0, INT32_MAX };
			st.currentBand[i] = 1;
		}
		const std::vector<Edge>& extras = st.queue.extras[i];
		Item& thisNode = currentSlice.at(i);
		WS oldEnd = thisNode.endSlice;
		if (!thisNode.exists) oldEnd = WS { 0, 0, INT32_MAX };
		const WS extra = st.hasSeedStart[i] ? seeds.slice : FakeSlice;
		if (!isFake(extra)) oldEnd = merge(oldEnd, extra);
		Item previousThisNode;
		if (st.previousBand[i])
		{
			previousThisNode = previousSlice.at(i);
			ORA_ASSERT(previousThisNode.exists);
		}
		else
		{
			previousThisNode.HP = AllOnes;
			previousThisNode.HN = 0;
			previousThisNode.exists = false;
		}
		NodeCalc nodeCalc = calcNode<true>(g, p, i, thisNode, eqv, previousThisNode, extras, &st.previousBand, (i32)j, nullptr, columnSteps, extra);
		ORA_ASSERT(nodeCalc.maxExactEndposScore != INT32_MIN);
		st.queue.pop();
		if (seeds.store) thisNode.nodeMax = std::max(nodeCalc.maxExactEndposScore, thisNode.nodeMax);
		ORA_ASSERT(nodeCalc.minScore <= (i32)j + bandwidth + 64 + 64);
		currentMinScoreAtEndRow = std::min(currentMinScoreAtEndRow, nodeCalc.minScore);
		if (nodeCalc.minScore < thisNode.minScore) thisNode.minScore = nodeCalc.minScore;
		WS newEnd = thisNode.endSlice;
		if (!(newEnd == oldEnd))
		{
			i32 newEndMinScore = changedMinScore(newEnd, oldEnd);
			ORA_ASSERT(newEndMinScore != INT32_MAX);
			if (newEndMinScore <= add(currentMinScoreAtEndRow, bandwidth))
			{
				for (const uint32_t* nb = g.outBegin(i); nb != g.outEnd(i); nb++)
				{
					st.queue.insert(g.d->component[*nb], newEndMinScore, Edge { *nb, newEnd, false });
				}
			}
		}
		if (nodeCalc.minScore < result.minScore)
		{
			result.minScore = nodeCalc.minScore;
			result.minScoreNode = nodeCalc.minScoreNode;
			result.minScoreNodeOffset = nodeCalc.minScoreNodeOffset;
		}
		if (nodeCalc.maxExactEndposScore > result.maxExactEndposScore)
		{
			result.maxExactEndposScore = nodeCalc.maxExactEndposScore;
			result.maxExactEndposNode = nodeCalc.maxExactEndposNode;
		}
		ORA_ASSERT(result.minScore == currentMinScoreAtEndRow);
		result.cellsProcessed += nodeCalc.cellsProcessed;
		ORA_ASSERT(nodeCalc.cellsProcessed > 0);
		if (result.cellsProcessed > p.maxCells) break;
	}
	for (size_t k = 0; k < seeds.count && multiseed; k++) st.hasSeedStart[seeds.nodes[k]] = 0;
	ORA_ASSERT(result.minScoreNode != SIZE_MAX || (multiseed && seeds.count == 0));
	st.queue.clear();
	return result;
}

struct Trace
{
	struct TItem { size_t node; size_t nodeOffset; size_t seqPos; bool nodeSwitch; };
	std::vector<TItem> items;
	i32 score = 0;
};

struct Pos
{
	size_t node, nodeOffset, seqPos;
	bool operator==(const Pos& o) const { return node == o.node && nodeOffset == o.nodeOffset && seqPos == o.seqPos; }
	bool operator!=(const Pos& o) const { return !(*this == o); }
};

static std::vector<WS> recalc(const Graph& g, const Params& p, uint32_t node, const Item& slice, const EqV& eqv, const Item& previous, i32 seqOffset,
	const WS& extra = FakeSlice)
{
	std::vector<Edge> incoming;
	incoming.push_back(Edge { node, slice.startSlice, true });
	std::vector<WS> result;
	result.reserve(64);
	Item copy = slice;
	uint64_t dummy = 0;
	calcNode<false>(g, p, node, copy, eqv, previous, incoming, nullptr, seqOffset, &result, dummy, extra);
	ORA_ASSERT(result.size() == g.len(node));
	ORA_ASSERT(result[0] == slice.startSlice);
	ORA_ASSERT(result.back() == slice.endSlice);
	return result;
}

static Item previousOrDefault(const Band& band, uint32_t node)
{
	if (band.has(node)) return band.at(node);
	Item r;
	r.HP = AllOnes;
	r.HN = 0;
	return r;
}

// pickBacktraceInside (Common.h:770-815)
static std::vector<Pos> backtraceInside(const Graph& g, size_t verticalOffset, const std::vector<WS>& ns, Pos pos, const char* seq, const WS& extra)
{
	size_t hori = pos.nodeOffset;
	size_t vert = pos.seqPos - verticalOffset;
	std::vector<Pos> result;
	while (hori > 0 && vert > 0)
	{
		i32 scoreHere = getValue(ns[hori], (int)vert);
		i32 verticalScore = getValue(ns[hori], (int)vert - 1);
		i32 horizontalScore = getValue(ns[hori - 1], (int)vert);
		i32 diagonalScore = getValue(ns[hori - 1], (int)vert - 1);
		bool eq = characterMatch(seq[vert + verticalOffset], g.charAt((uint32_t)pos.node, (uint32_t)hori));
		if (verticalScore == scoreHere - 1) { vert--; result.push_back(Pos { pos.node, hori, vert + verticalOffset }); continue; }
		if (diagonalScore == scoreHere - (eq ? 0 : 1)) { hori--; vert--; result.push_back(Pos { pos.node, hori, vert + verticalOffset }); continue; }
		if (horizontalScore == scoreHere - 1) { hori--; result.push_back(Pos { pos.node, hori, vert + verticalOffset }); continue; }
		ORA_ASSERT(scoreHere == getValue(extra, (int)vert));
		break;
	}
	return result;
}

struct Step { Pos pos; bool nodeSwitch; };

// pickBacktraceCorner (Common.h:936-1054)
static Step backtraceCorner(const Graph& g, const Band& current, const Band& previous, uint32_t node, size_t j, const char* seq,
	i32 quitScore, bool scoresNotValid, i32 previousQuitScore, bool previousScoresNotValid, const WS& extra)
{
	i32 scoreHere = getValue(current.at(node).startSlice, 0);
	if (scoresNotValid || scoreHere > quitScore)
	{
		if (scoreHere == getValue(extra, 0)) return Step { Pos { node, 0, j }, false };
		i32 smallestFound = scoreHere + 1;
		Pos smallestPos { SIZE_MAX, SIZE_MAX, SIZE_MAX };
		bool nodeChange = false;
		if (previous.has(node))
		{
			smallestFound = previous.at(node).startSlice.scoreEnd;
			smallestPos = Pos { node, 0, j - 1 };
			nodeChange = false;
		}
		for (const uint32_t* nbp = g.inBegin(node); nbp != g.inEnd(node); nbp++)
		{
			uint32_t nb = *nbp;
			if (previous.has(nb))
			{
				WS ns = previous.at(nb).endSlice;
				if (ns.scoreEnd <= smallestFound)
				{
					smallestFound = ns.scoreEnd;
					smallestPos = Pos { nb, g.len(nb) - 1u, j - 1 };
					nodeChange = true;
				}
			}
			if (current.has(nb) && nb != node)
			{
				WS ns = current.at(nb).endSlice;
				if (getValue(ns, 0) < smallestFound)
				{
					smallestFound = getValue(ns, 0);
					smallestPos = Pos { nb, g.len(nb) - 1u, j };
					nodeChange = true;
				}
			}
		}
		ORA_ASSERT(smallestPos.node != SIZE_MAX);
		return Step { smallestPos, nodeChange };
	}
	bool eq = characterMatch(seq[j], g.charAt(node, 0));
	Pos bestInvalid { SIZE_MAX, SIZE_MAX, SIZE_MAX };
	i32 bestInvalidScore = scoreHere + 1;
	bool bestInvalidSwitch = false;
	if (previous.has(node))
	{
		i32 ps = previous.at(node).startSlice.scoreEnd;
		ORA_ASSERT(ps >= scoreHere - 1);
		if (ps == scoreHere - 1) return Step { Pos { node, 0, j - 1 }, false };
		if (previousScoresNotValid || ps > previousQuitScore)
		{
			if (ps < bestInvalidScore)
			{
				bestInvalidScore = ps;
				bestInvalid = Pos { node, 0, j - 1 };
				bestInvalidSwitch = false;
			}
		}
	}
	for (const uint32_t* nbp = g.inBegin(node); nbp != g.inEnd(node); nbp++)
	{
		uint32_t nb = *nbp;
		if (current.has(nb))
		{
			i32 v = getValue(current.at(nb).endSlice, 0);
			ORA_ASSERT(v >= scoreHere - 1);
			if (v == scoreHere - 1) return Step { Pos { nb, g.len(nb) - 1u, j }, true };
		}
		if (previous.has(nb))
		{
			i32 cornerScore = previous.at(nb).endSlice.scoreEnd;
			if (previousScoresNotValid || cornerScore > previousQuitScore)
			{
				if (cornerScore < bestInvalidScore)
				{
					bestInvalidScore = cornerScore;
					bestInvalid = Pos { nb, g.len(nb) - 1u, j - 1 };
					bestInvalidSwitch = true;
				}
			}
			else
			{
				ORA_ASSERT(cornerScore >= scoreHere - (eq ? 0 : 1));
				if (cornerScore == scoreHere - (eq ? 0 : 1)) return Step { Pos { nb, g.len(nb) - 1u, j - 1 }, true };
			}
		}
	}
	if (eq && scoreHere == scoreBeforeStart(extra)) return Step { Pos { node, 0, j }, false };
	if (scoreHere == getValue(extra, 0)) return Step { Pos { node, 0, j }, false };
	if (bestInvalidScore < scoreHere + 1) return Step { bestInvalid, bestInvalidSwitch };
	ORA_ASSERT(false);
	return Step { Pos { 0, 0, 0 }, false };
}

// pickBacktraceHorizontalCrossing (Common.h:817-884): returns (walked-to position, next step)
static std::pair<Step, Step> backtraceHorizontal(const Graph& g, const Band& current, const Band& previous, size_t j, uint32_t node, Pos pos,
	const char* seq, i32 quitScore, bool scoresNotValid, i32 previousQuitScore, bool previousScoresNotValid, const WS& extra)
{
	WS startSlice = current.at(node).startSlice;
	while (pos.seqPos % 64 != 0 && (startSlice.VP & (1ULL << (pos.seqPos % 64)))) pos.seqPos--;
	size_t offset = pos.seqPos % 64;
	if (offset == 0) return { Step { pos, false }, backtraceCorner(g, current, previous, node, j, seq, quitScore, scoresNotValid, previousQuitScore, previousScoresNotValid, extra) };
	bool eq = characterMatch(seq[pos.seqPos], g.charAt((uint32_t)pos.node, (uint32_t)pos.nodeOffset));
	i32 scoreHere = getValue(startSlice, (int)offset);
	if (scoresNotValid || scoreHere > quitScore)
	{
		i32 smallestFound = getValue(startSlice, (int)offset - 1);
		Pos smallestPos { node, 0, pos.seqPos - 1 };
		bool nodeChange = false;
		for (const uint32_t* nbp = g.inBegin(node); nbp != g.inEnd(node); nbp++)
		{
			uint32_t nb = *nbp;
			if (current.has(nb))
			{
				WS ns = current.at(nb).endSlice;
				if (getValue(ns, (int)offset - 1) <= smallestFound)
				{
					smallestFound = getValue(ns, (int)offset - 1);
					smallestPos = Pos { nb, g.len(nb) - 1u, pos.seqPos - 1 };
					nodeChange = true;
				}
				if (getValue(ns, (int)offset) < smallestFound && nb != node)
				{
					smallestFound = getValue(ns, (int)offset);
					smallestPos = Pos { nb, g.len(nb) - 1u, pos.seqPos };
					nodeChange = true;
				}
			}
		}
		if (smallestPos == pos) ORA_ASSERT(getValue(extra, (int)offset) == scoreHere);
		return { Step { pos, false }, Step { smallestPos, nodeChange } };
	}
	for (const uint32_t* nbp = g.inBegin(node); nbp != g.inEnd(node); nbp++)
	{
		uint32_t nb = *nbp;
		if (current.has(nb))
		{
			WS ns = current.at(nb).endSlice;
			ORA_ASSERT(getValue(ns, (int)offset) >= scoreHere - 1);
			ORA_ASSERT(getValue(ns, (int)offset - 1) >= scoreHere - (eq ? 0 : 1));
			if (getValue(ns, (int)offset) == scoreHere - 1) return { Step { pos, false }, Step { Pos { nb, g.len(nb) - 1u, pos.seqPos }, true } };
			if (getValue(ns, (int)offset - 1) == scoreHere - (eq ? 0 : 1)) return { Step { pos, false }, Step { Pos { nb, g.len(nb) - 1u, pos.seqPos - 1 }, true } };
		}
	}
	ORA_ASSERT(scoreHere == getValue(extra, (int)offset));
	return { Step { pos, false }, Step { pos, false } };
}

// pickBacktraceVerticalCrossing (Common.h:886-934)
static std::pair<Step, Step> backtraceVertical(const Graph& g, const Band& current, const Band& previous, const std::vector<WS>& ns, size_t j,
	uint32_t node, Pos pos, const char* seq, i32 quitScore, bool scoresNotValid, i32 previousQuitScore, bool previousScoresNotValid,
	const WS& extra)
{
	ORA_ASSERT(pos.nodeOffset > 0);
	while (pos.nodeOffset > 0 && getValue(ns[pos.nodeOffset - 1], 0) == getValue(ns[pos.nodeOffset], 0) - 1) pos.nodeOffset--;
	if (pos.nodeOffset == 0) return { Step { pos, false }, backtraceCorner(g, current, previous, node, j, seq, quitScore, scoresNotValid, previousQuitScore, previousScoresNotValid, extra) };
	ORA_ASSERT(previous.has(node));
	bool eq = characterMatch(seq[pos.seqPos], g.charAt((uint32_t)pos.node, (uint32_t)pos.nodeOffset));
	const Item& previousNode = previous.at(node);
	i32 scoreHere = getValue(ns[pos.nodeOffset], 0);
	i32 scoreDiagonal = previousNode.startSlice.scoreEnd;
	for (size_t i = 1; i <= pos.nodeOffset - 1; i++)
	{
		scoreDiagonal += (previousNode.HP >> i) & 1;
		scoreDiagonal -= (previousNode.HN >> i) & 1;
	}
	i32 scoreUp = scoreDiagonal;
	scoreUp += (previousNode.HP >> pos.nodeOffset) & 1;
	scoreUp -= (previousNode.HN >> pos.nodeOffset) & 1;
	if (previousScoresNotValid || scoresNotValid || scoreHere > quitScore || scoreDiagonal > previousQuitScore || scoreUp > previousQuitScore)
	{
		if (scoreHere == getValue(extra, 0)) return { Step { pos, false }, Step { pos, false } };
		if (scoreDiagonal < scoreUp) return { Step { pos, false }, Step { Pos { pos.node, pos.nodeOffset - 1, pos.seqPos - 1 }, false } };
		return { Step { pos, false }, Step { Pos { pos.node, pos.nodeOffset, pos.seqPos - 1 }, false } };
	}
	ORA_ASSERT(scoreUp >= scoreHere - 1);
	ORA_ASSERT(scoreDiagonal >= scoreHere - (eq ? 0 : 1));
	if (scoreUp == scoreHere - 1) return { Step { pos, false }, Step { Pos { pos.node, pos.nodeOffset, pos.seqPos - 1 }, false } };
	if (scoreDiagonal == scoreHere - (eq ? 0 : 1)) return { Step { pos, false }, Step { Pos { pos.node, pos.nodeOffset - 1, pos.seqPos - 1 }, false } };
	ORA_ASSERT(scoreHere == getValue(extra, 0));
	return { Step { pos, false }, Step { pos, false } };
}

static void checkCircularity(const Trace& t)   // checkBacktraceCircularity (Common.h:760-768)
{
	const auto& b = t.items.back();
	for (size_t i = t.items.size() - 2; i < t.items.size(); i--)
	{
		const auto& x = t.items[i];
		ORA_ASSERT(!(x.node == b.node && x.nodeOffset == b.nodeOffset && x.seqPos == b.seqPos));
		if (x.seqPos != b.seqPos) return;
	}
}

// getSeedSlice (Common.h:320-353): the column of starting an alignment at each row of the
// slice at j, scored as the X-score's error cost of the skipped read prefix
static WS seedSlice(size_t j, size_t seqLen, i32 cost)
{
	ORA_ASSERT(j % 64 == 0);
	WS r { 0, 0, 0 };
	i32 oldSeedScore = 0;
	if (j > 0) oldSeedScore = ((i32)(j - 1 + 1) * 100 + cost / 2) / cost;
	for (size_t offset = 0; offset < 64; offset++)
	{
		if (j + offset >= seqLen)
		{
			r.VP |= 1ULL << offset;
			oldSeedScore = oldSeedScore + 1;
			continue;
		}
		i32 seedScore = ((i32)(j + offset + 1) * 100 + cost / 2) / cost;
		ORA_ASSERT(seedScore == oldSeedScore || seedScore == oldSeedScore + 1);
		if (seedScore == oldSeedScore + 1) r.VP |= 1ULL << offset;
		oldSeedScore = seedScore;
	}
	r.scoreEnd = oldSeedScore;
	r.VP &= ~1ULL;
	r.VN |= 1;
	return r;
}

// getReverseTraceFromTable (Common.h:571-758).  multiseed: a node that is a seed start in its
// slice is recomputed and backtracked with the seed-start slice as extraSlice, and the walk
// along the row above the read (:721-756) is skipped.
static Trace traceFromTable(const Graph& g, const Params& p, const char* seq, size_t seqLen, const std::vector<Slice>& table, Pos startPos, i32 startScore,
	bool multiseed = false)
{
	ORA_ASSERT(table.size() > 0);
	size_t currentSlice = startPos.seqPos / 64 + 1;
	ORA_ASSERT(currentSlice < table.size());
	Trace result;
	result.score = startScore;
	result.items.push_back({ startPos.node, startPos.nodeOffset, startPos.seqPos, false });
	size_t currentNode = SIZE_MAX;
	std::vector<WS> nodeSlices;
	EqV eqv = getEq(seq, seqLen, (size_t)table[currentSlice].j);
	i32 lastScore = INT32_MAX - 1;
	WS extra = FakeSlice;
	auto back = [&]() -> Pos { const auto& b = result.items.back(); return Pos { b.node, b.nodeOffset, b.seqPos }; };
	auto push = [&](Pos q, bool sw) { result.items.push_back({ q.node, q.nodeOffset, q.seqPos, sw }); };
	while (result.items.back().seqPos != (size_t)-1)
	{
		Pos b = back();
		size_t newSlice = b.seqPos / 64 + 1;
		ORA_ASSERT(newSlice < table.size());
		size_t newNode = b.node;
		if (newSlice != currentSlice || newNode != currentNode)
		{
			if (newSlice != currentSlice) eqv = getEq(seq, seqLen, (size_t)table[newSlice].j);
			currentSlice = newSlice;
			currentNode = newNode;
			ORA_ASSERT(table[currentSlice].scores.has((uint32_t)currentNode));
			ORA_ASSERT(currentSlice > 0);
			Item previous = previousOrDefault(table[currentSlice - 1].scores, (uint32_t)currentNode);
			const Item& here = table[currentSlice].scores.at((uint32_t)currentNode);
			extra = here.seedStart ? seedSlice((size_t)table[currentSlice].j, seqLen, p.cost) : FakeSlice;
			nodeSlices = recalc(g, p, (uint32_t)currentNode, here, eqv, previous, (i32)table[currentSlice].j, extra);
		}
		const Slice& cs = table[currentSlice];
		const Slice& ps = table[currentSlice - 1];
		i32 quit = add(cs.minScore, (i32)cs.bandwidth);
		i32 pquit = add(ps.minScore, (i32)ps.bandwidth);
		ORA_ASSERT(b.nodeOffset < g.len((uint32_t)currentNode));
		lastScore = getValue(nodeSlices[b.nodeOffset], (int)(b.seqPos % 64));
		if (b.seqPos % 64 == 0 && b.nodeOffset == 0)
		{
			Step bt = backtraceCorner(g, cs.scores, ps.scores, (uint32_t)currentNode, (size_t)cs.j, seq, quit, cs.scoresNotValid, pquit, ps.scoresNotValid, extra);
			if (bt.pos == b && !bt.nodeSwitch && getValue(nodeSlices[bt.pos.nodeOffset], (int)(bt.pos.seqPos % 64)) == getValue(extra, (int)(bt.pos.seqPos % 64))) break;
			if (bt.pos == b && !bt.nodeSwitch && getValue(nodeSlices[bt.pos.nodeOffset], (int)(bt.pos.seqPos % 64)) == scoreBeforeStart(extra)) break;
			push(bt.pos, bt.nodeSwitch);
			checkCircularity(result);
			continue;
		}
		if (b.seqPos % 64 == 0)
		{
			ORA_ASSERT(b.nodeOffset > 0);
			if (!ps.scores.has((uint32_t)currentNode))
			{
				for (size_t i = b.nodeOffset - 1; i > 0; i--) push(Pos { currentNode, i, b.seqPos }, false);
				push(Pos { currentNode, 0, b.seqPos }, false);
				continue;
			}
			auto crossing = backtraceVertical(g, cs.scores, ps.scores, nodeSlices, (size_t)cs.j, (uint32_t)currentNode, b, seq, quit, cs.scoresNotValid, pquit, ps.scoresNotValid, extra);
			if (crossing.second.pos.seqPos == b.seqPos && getValue(nodeSlices[crossing.second.pos.nodeOffset], (int)(crossing.second.pos.seqPos % 64)) == getValue(extra, (int)(crossing.second.pos.seqPos % 64))) break;
			ORA_ASSERT(crossing.first.pos.node == b.node);
			ORA_ASSERT(crossing.first.pos.seqPos == b.seqPos);
			ORA_ASSERT(crossing.first.pos.nodeOffset <= b.nodeOffset);
			if (crossing.first.pos.nodeOffset != b.nodeOffset)
			{
				for (size_t off = b.nodeOffset - 1; off != crossing.first.pos.nodeOffset; off--) push(Pos { crossing.first.pos.node, off, crossing.first.pos.seqPos }, false);
			}
			if (crossing.first.pos != back()) push(crossing.first.pos, crossing.first.nodeSwitch);
			ORA_ASSERT(crossing.second.pos != back());
			push(crossing.second.pos, crossing.second.nodeSwitch);
			continue;
		}
		if (b.nodeOffset == 0)
		{
			auto crossing = backtraceHorizontal(g, cs.scores, ps.scores, (size_t)cs.j, (uint32_t)currentNode, b, seq, quit, cs.scoresNotValid, pquit, ps.scoresNotValid, extra);
			if (crossing.second.pos.node == b.node && !crossing.second.nodeSwitch && getValue(nodeSlices[crossing.second.pos.nodeOffset], (int)(crossing.second.pos.seqPos % 64)) == getValue(extra, (int)(crossing.second.pos.seqPos % 64))) break;
			ORA_ASSERT(crossing.first.pos.node == b.node);
			ORA_ASSERT(crossing.first.pos.nodeOffset == b.nodeOffset);
			ORA_ASSERT(crossing.first.pos.seqPos <= b.seqPos);
			if (crossing.first.pos.seqPos != b.seqPos)
			{
				for (size_t sp = b.seqPos - 1; sp != crossing.first.pos.seqPos; sp--) push(Pos { crossing.first.pos.node, crossing.first.pos.nodeOffset, sp }, false);
			}
			if (crossing.first.pos != back()) push(crossing.first.pos, crossing.first.nodeSwitch);
			ORA_ASSERT(crossing.second.pos != back());
			push(crossing.second.pos, crossing.second.nodeSwitch);
			checkCircularity(result);
			continue;
		}
		auto inner = backtraceInside(g, (size_t)cs.j, nodeSlices, b, seq, extra);
		for (const auto& q : inner) push(q, false);
		Pos nb = back();
		if (getValue(nodeSlices[nb.nodeOffset], (int)(nb.seqPos % 64)) == getValue(extra, (int)(nb.seqPos % 64))) break;
	}
	ORA_ASSERT(result.score >= lastScore);
	result.score -= lastScore;
	// walk along the start node's row above the read (Common.h:721-756)
	if (!multiseed)
	{
		Pos b = back();
		ORA_ASSERT(b.seqPos == (size_t)-1);
		const Item& node = table[0].scores.at((uint32_t)b.node);
		uint32_t L = g.len((uint32_t)b.node);
		std::vector<i32> before(L);
		before[0] = node.startSlice.scoreEnd;
		for (uint32_t i = 1; i < L; i++) before[i] = before[i - 1] + (i32)((node.HP >> i) & 1) - (i32)((node.HN >> i) & 1);
		ORA_ASSERT(before.back() == node.endSlice.scoreEnd);
		while (before[back().nodeOffset] != 0 && back().nodeOffset > 0 && before[back().nodeOffset - 1] == before[back().nodeOffset] - 1)
		{
			Pos q = back();
			push(Pos { q.node, q.nodeOffset - 1, q.seqPos }, false);
		}
		Pos q = back();
		if (q.nodeOffset == 0 && before[q.nodeOffset] != 0)
		{
			for (const uint32_t* nbp = g.inBegin((uint32_t)q.node); nbp != g.inEnd((uint32_t)q.node); nbp++)
			{
				uint32_t nbn = *nbp;
				if (table[0].scores.has(nbn) && scoreBeforeStart(table[0].scores.at(nbn).endSlice) == before[q.nodeOffset] - 1)
				{
					push(Pos { nbn, g.len(nbn) - 1u, q.seqPos }, true);
					break;
				}
			}
		}
	}
	return result;
}

// getReverseTraceFromTableExactEndPos (Common.h:496-562)
static Trace traceExactEndPos(const Graph& g, const Params& p, const char* seq, size_t seqLen, const std::vector<Slice>& table)
{
	ORA_ASSERT(table.size() > 1);
	size_t bestIndex = 1;
	for (size_t i = 1; i < table.size(); i++)
	{
		if (table[i].maxExactEndposScore > table[bestIndex].maxExactEndposScore) bestIndex = i;
	}
	uint32_t node = (uint32_t)table[bestIndex].maxExactEndposNode;
	i32 score = table[bestIndex].maxExactEndposScore;
	Item previous = previousOrDefault(table[bestIndex - 1].scores, node);
	size_t j = (size_t)table[bestIndex].j;
	EqV eqv = getEq(seq, seqLen, j);
	std::vector<WS> ns = recalc(g, p, node, table[bestIndex].scores.at(node), eqv, previous, (i32)j);
	size_t nodeOffset = SIZE_MAX;
	size_t bvOffset = SIZE_MAX;
	int cells = (int)std::min<size_t>(64, seqLen - j);
	for (size_t i = 0; i < ns.size(); i++)
	{
		i32 maxScore = maxXScore(ns[i], (i32)j, p.cost, cells);
		ORA_ASSERT(maxScore <= score);
		if (maxScore == score)
		{
			for (size_t off = 63; off < 64; off--)
			{
				if (j + off >= seqLen) continue;
				i32 scoreHere = getXScore(ns[i], (i32)j, (int)off, p.cost);
				ORA_ASSERT(scoreHere <= score);
				if (scoreHere == score)
				{
					if (nodeOffset == SIZE_MAX || off > bvOffset)
					{
						nodeOffset = i;
						bvOffset = off;
					}
				}
			}
		}
	}
	ORA_ASSERT(nodeOffset != SIZE_MAX);
	ORA_ASSERT(bvOffset != SIZE_MAX);
	ORA_ASSERT(j + bvOffset < seqLen);
	i32 startScore = getValue(ns[nodeOffset], (int)bvOffset);
	return traceFromTable(g, p, seq, seqLen, table, Pos { node, nodeOffset, j + bvOffset }, startScore);
}

// getReverseTraceFromSeed (GraphAlignerBitvectorBanded.h:59-76) with getInitialSliceExactPosition
// (Common.h:1551-1587) and getXdropSlices (Banded.h:580-725).
static int extendOne(const Graph& g, const Params& p, const char* seq, size_t seqLen, uint32_t startNode, uint32_t offsetInNode,
	State& st, Trace& out, uint64_t& columnSteps)
{
	size_t numSlices = (seqLen + 63) / 64;
	std::vector<Slice> table;
	table.reserve(numSlices + 1);
	Slice init;
	init.j = -64;
	init.bandwidth = 1;
	init.minScore = 0;
	ORA_ASSERT(startNode < g.d->num_nodes && offsetInNode < g.len(startNode));
	init.minScoreNode = startNode;
	init.minScoreNodeOffset = offsetInNode;
	init.maxExactEndposScore = 0;
	init.maxExactEndposNode = startNode;
	{
		Item& node = init.scores.add(startNode);
		node.startSlice = WS { 0, 0, (i32)offsetInNode };
		node.endSlice = WS { 0, 0, (i32)g.len(startNode) - 1 - (i32)offsetInNode };
		node.minScore = 0;
		node.exists = true;
		for (uint32_t i = 1; i <= offsetInNode; i++) node.HN |= 1ULL << i;
		for (uint32_t i = offsetInNode + 1; i < g.len(startNode); i++) node.HP |= 1ULL << i;
	}
	table.push_back(init);
	for (auto n : init.scores.nodes) st.previousBand[n] = 1;
	i32 bestXScore = init.maxExactEndposScore;
	size_t lastIndex = 0;    // table index of lastSlice
	for (size_t s = 0; s < numSlices; s++)
	{
		const Slice& lastSlice = table[lastIndex];
		Slice newSlice;
		newSlice.j = lastSlice.j + 64;
		NodeCalc r = calculateSlice(g, p, seq, seqLen, (size_t)newSlice.j, newSlice.scores, lastSlice.scores, st,
			add(lastSlice.minScore, (i32)lastSlice.bandwidth), (int)p.bandwidth, lastSlice.minScore, columnSteps);
		newSlice.cellsProcessed = r.cellsProcessed;
		newSlice.minScoreNode = r.minScoreNode;
		newSlice.minScoreNodeOffset = r.minScoreNodeOffset;
		newSlice.minScore = r.minScore;
		newSlice.maxExactEndposScore = r.maxExactEndposScore;
		newSlice.maxExactEndposNode = r.maxExactEndposNode;
		newSlice.bandwidth = p.bandwidth;
		ORA_ASSERT(newSlice.minScore != INT32_MAX);
		ORA_ASSERT(newSlice.minScoreNode != SIZE_MAX);
		ORA_ASSERT(newSlice.scores.has((uint32_t)newSlice.minScoreNode));
		ORA_ASSERT(newSlice.maxExactEndposScore != INT32_MIN);
		if (newSlice.maxExactEndposScore > bestXScore) bestXScore = newSlice.maxExactEndposScore;
		if (newSlice.cellsProcessed >= p.maxCells) newSlice.scoresNotValid = true;
		if ((double)newSlice.maxExactEndposScore < (double)bestXScore - (double)p.xdrop)
		{
			for (auto n : lastSlice.scores.nodes) st.previousBand[n] = 0;
			for (auto n : newSlice.scores.nodes) st.currentBand[n] = 0;
			break;
		}
		for (auto n : lastSlice.scores.nodes) st.previousBand[n] = 0;
		ORA_ASSERT(newSlice.minScore >= lastSlice.minScore);
		table.push_back(std::move(newSlice));
		lastIndex = table.size() - 1;
		if (s == numSlices - 1)
		{
			for (auto n : table.back().scores.nodes) st.currentBand[n] = 0;
		}
		else
		{
			std::swap(st.previousBand, st.currentBand);
		}
	}
	if (table.size() <= 1) return GA_TRACE_FAILED;
	out = traceExactEndPos(g, p, seq, seqLen, table);
	return GA_OK;
}

// GraphAlignerBitvectorBanded::getMultiseedSlices (GraphAlignerBitvectorBanded.h:727-822): every
// slice of the read from the empty initial slice, the seeds of each slice started in it.
// seedSlices/seedNodes: the read's seeds in slice order (prepareSeedsForMultiseeding).
static std::vector<Slice> multiseedFill(const Graph& g, const Params& p, const char* seq, size_t seqLen, const uint32_t* seedSlices,
	const uint32_t* seedNodes, size_t numSeeds, State& st, uint64_t& columnSteps)
{
	const size_t numSlices = (seqLen + 63) / 64;
	std::vector<Slice> table;
	table.reserve(numSlices + 1);
	Slice init;    // getInitialEmptySlice (Common.h:1541-1549)
	init.j = -64;
	init.bandwidth = 1;
	init.minScore = 0;
	table.push_back(init);
	size_t lastSeedHit = 0;
	try
	{
		for (size_t s = 0; s < numSlices; s++)
		{
			const Slice& lastSlice = table.back();
			const size_t sliceIndex = (size_t)(lastSlice.j + 64) / 64;
			size_t nextSeedHit = lastSeedHit;
			ORA_ASSERT(nextSeedHit == numSeeds || seedSlices[nextSeedHit] >= sliceIndex);
			while (nextSeedHit < numSeeds && seedSlices[nextSeedHit] == sliceIndex) nextSeedHit++;
			Slice newSlice;
			newSlice.j = lastSlice.j + 64;
			SliceSeeds seeds;
			seeds.nodes = seedNodes + lastSeedHit;
			seeds.count = nextSeedHit - lastSeedHit;
			seeds.slice = seedSlice((size_t)newSlice.j, seqLen, p.cost);
			seeds.store = true;
			NodeCalc r = calculateSlice(g, p, seq, seqLen, (size_t)newSlice.j, newSlice.scores, lastSlice.scores, st,
				add(lastSlice.minScore, (i32)lastSlice.bandwidth), (int)p.bandwidth, lastSlice.minScore, columnSteps, seeds);
			lastSeedHit = nextSeedHit;
			newSlice.cellsProcessed = r.cellsProcessed;
			newSlice.minScoreNode = r.minScoreNode;
			newSlice.minScoreNodeOffset = r.minScoreNodeOffset;
			newSlice.minScore = r.minScore;
			newSlice.maxExactEndposScore = r.maxExactEndposScore;
			newSlice.maxExactEndposNode = r.maxExactEndposNode;
			newSlice.bandwidth = p.bandwidth;
			if (newSlice.cellsProcessed >= p.maxCells) newSlice.scoresNotValid = true;
			for (auto n : lastSlice.scores.nodes) st.previousBand[n] = 0;
			table.push_back(std::move(newSlice));
			if (s == numSlices - 1)
			{
				for (auto n : table.back().scores.nodes) st.currentBand[n] = 0;
			}
			else
			{
				std::swap(st.previousBand, st.currentBand);
			}
		}
		ORA_ASSERT(lastSeedHit == numSeeds);
	}
	catch (...)
	{
		// leave the per-graph flags clear for the next read
		for (const auto& sl : table)
			for (auto n : sl.scores.nodes) st.previousBand[n] = st.currentBand[n] = st.hasSeedStart[n] = 0;
		throw;
	}
	return table;
}

// GraphAlignerBitvectorCommon::getLocalMaximaTracesFromTable (Common.h:355-494) with
// sliceConsistency and multiseed: a trace from every node whose best exact-end-position
// X-score in a slice is a local maximum over the slices above and below and the node's
// neighbours, in slice order from the last and band order within a slice.
static std::vector<Trace> localMaximaTraces(const Graph& g, const Params& p, const char* seq, size_t seqLen, const std::vector<Slice>& table)
{
	std::vector<Trace> result;
	ORA_ASSERT(table.size() > 1);
	ORA_ASSERT(table[0].scores.size() == 0);
	std::vector<i32> sliceMaxScores(table.size());
	for (size_t i = 0; i < table.size(); i++) sliceMaxScores[i] = table[i].maxExactEndposScore;
	auto maxOf = [&](size_t slice, uint32_t node, i32& out) -> bool
	{
		if (!table[slice].scores.has(node)) return false;
		out = table[slice].scores.at(node).nodeMax;
		return true;
	};
	for (size_t currentSlice = table.size() - 1; currentSlice > 0; currentSlice--)
	{
		const Slice& cs = table[currentSlice];
		if (cs.maxExactEndposScore <= 0) continue;
		for (size_t k = 0; k < cs.scores.size(); k++)
		{
			const uint32_t node = cs.scores.nodes[k];
			const Item& item = cs.scores.items[k];
			if (!item.exists) continue;
			const i32 score = item.nodeMax;
			if (score <= 0) continue;
			if (score < sliceMaxScores[currentSlice] * p.multimapScoreFraction) continue;
			i32 other;
			if (maxOf(currentSlice - 1, node, other) && other > score) continue;
			if (currentSlice < table.size() - 1 && maxOf(currentSlice + 1, node, other) && other >= score) continue;
			bool notLocalMaximum = false;
			for (const uint32_t* nb = g.inBegin(node); nb != g.inEnd(node) && !notLocalMaximum; nb++)
			{
				if (maxOf(currentSlice, *nb, other) && other > score) notLocalMaximum = true;
				else if (maxOf(currentSlice - 1, *nb, other) && other > score) notLocalMaximum = true;
			}
			for (const uint32_t* nb = g.outBegin(node); nb != g.outEnd(node) && !notLocalMaximum; nb++)
			{
				if (maxOf(currentSlice, *nb, other) && other > score) notLocalMaximum = true;
				else if (currentSlice < table.size() - 1 && maxOf(currentSlice + 1, *nb, other) && other > score) notLocalMaximum = true;
			}
			if (notLocalMaximum) continue;
			Item previous = previousOrDefault(table[currentSlice - 1].scores, node);
			const size_t j = (size_t)cs.j;
			EqV eqv = getEq(seq, seqLen, j);
			const WS extra = item.seedStart ? seedSlice(j, seqLen, p.cost) : FakeSlice;
			std::vector<WS> ns = recalc(g, p, node, item, eqv, previous, (i32)j, extra);
			size_t nodeOffset = SIZE_MAX;
			size_t bvOffset = SIZE_MAX;
			int cells = (int)std::min<size_t>(64, seqLen - j);
			for (size_t i = 0; i < ns.size(); i++)
			{
				i32 maxScore = maxXScore(ns[i], (i32)j, p.cost, cells);
				ORA_ASSERT(maxScore <= score);
				if (maxScore != score) continue;
				for (size_t off = 63; off < 64; off--)
				{
					if (j + off >= seqLen) continue;
					i32 scoreHere = getXScore(ns[i], (i32)j, (int)off, p.cost);
					ORA_ASSERT(scoreHere <= score);
					if (scoreHere == score && (nodeOffset == SIZE_MAX || off > bvOffset))
					{
						nodeOffset = i;
						bvOffset = off;
					}
				}
			}
			ORA_ASSERT(nodeOffset != SIZE_MAX && bvOffset != SIZE_MAX);
			ORA_ASSERT(j + bvOffset < seqLen);
			i32 startScore = getValue(ns[nodeOffset], (int)bvOffset);
			result.push_back(traceFromTable(g, p, seq, seqLen, table, Pos { node, nodeOffset, j + bvOffset }, startScore, true));
			const size_t traceEnd = result.back().items[0].seqPos;
			const size_t traceStart = result.back().items.back().seqPos;
			ORA_ASSERT(traceEnd >= traceStart);
			const size_t startSlice = (size_t)(((double)(traceEnd - traceStart) * 0.05 + (double)traceStart + 64 - 1) / 64 + 1);
			for (size_t i = startSlice; i < currentSlice; i++) sliceMaxScores[i] = std::max(sliceMaxScores[i], score);
		}
	}
	return result;
}

}

static inline uint64_t packItem(size_t node, size_t nodeOffset, size_t seqPos, bool sw)
{
	uint64_t sp1 = (seqPos == (size_t)-1) ? 0 : (uint64_t)seqPos + 1;
	return (uint64_t)(uint32_t)node | ((uint64_t)(nodeOffset & 63) << 32) | ((uint64_t)(sw ? 1 : 0) << 38) | (sp1 << 39);
}

extern "C" int ora_extend_batch(const ga_graph_desc* graph, const ga_extend_params* params, const ga_extend_batch_desc* batch,
	ga_extend_results* results, int threads)
{
	if (!graph || !params || !batch || !results) return GA_ERR_ARGUMENT;
	ora::Graph g { graph };
	ora::Params p { params->bandwidth, params->xdrop, (size_t)params->max_cells_per_slice, params->xscore_error_cost };
	if (threads < 1) threads = 1;
	std::atomic<uint32_t> next { 0 };
	auto worker = [&]()
	{
		ora::State st { graph->num_nodes };
		while (true)
		{
			uint32_t i = next.fetch_add(1);
			if (i >= batch->num) break;
			ora::Trace trace;
			uint64_t steps = 0;
			int status;
			try
			{
				status = ora::extendOne(g, p, (const char*)batch->seq + batch->seq_offset[i], batch->seq_len[i], batch->start_node[i], batch->start_offset[i], st, trace, steps);
			}
			catch (const ora::AssertFail&)
			{
				status = GA_ASSERT;
				st = ora::State { graph->num_nodes };
			}
			if (results->cell_steps) results->cell_steps[i] = steps;
			results->status[i] = status;
			results->score[i] = status == GA_OK ? trace.score : 0;
			uint32_t n = 0;
			if (status == GA_OK)
			{
				if (trace.items.size() > batch->trace_capacity[i])
				{
					results->status[i] = GA_CAPACITY;
				}
				else
				{
					uint64_t* dst = results->trace_items + batch->trace_offset[i];
					for (const auto& t : trace.items) dst[n++] = packItem(t.node, t.nodeOffset, t.seqPos, t.nodeSwitch);
				}
			}
			results->trace_len[i] = n;
		}
	};
	std::vector<std::thread> pool;
	for (int t = 1; t < threads; t++) pool.emplace_back(worker);
	worker();
	for (auto& t : pool) t.join();
	return GA_OK;
}

// The multiseed DP of ga_multiseed_batch (include/graphaligner_gb300.h) on `threads` host threads:
// multiseedFill + localMaximaTraces per read.
extern "C" int ora_multiseed_batch(const ga_graph_desc* graph, const ga_extend_params* params, const ga_multiseed_batch_desc* batch,
	ga_multiseed_results* results, int threads)
{
	if (!graph || !params || !batch || !results) return GA_ERR_ARGUMENT;
	ora::Graph g { graph };
	ora::Params p { params->bandwidth, params->xdrop, (size_t)params->max_cells_per_slice, params->xscore_error_cost, batch->multimap_score_fraction };
	if (threads < 1) threads = 1;
	std::atomic<uint32_t> next { 0 };
	auto worker = [&]()
	{
		ora::State st { graph->num_nodes };
		while (true)
		{
			uint32_t i = next.fetch_add(1);
			if (i >= batch->num) break;
			const uint64_t s0 = batch->seed_offset[i], s1 = batch->seed_offset[i + 1];
			std::vector<ora::Trace> traces;
			uint64_t steps = 0;
			int status = GA_OK;
			try
			{
				auto table = ora::multiseedFill(g, p, (const char*)batch->seq + batch->seq_offset[i], batch->seq_len[i], batch->seed_slice + s0,
					batch->seed_node + s0, (size_t)(s1 - s0), st, steps);
				traces = ora::localMaximaTraces(g, p, (const char*)batch->seq + batch->seq_offset[i], batch->seq_len[i], table);
			}
			catch (const ora::AssertFail&)
			{
				status = GA_ASSERT;
				st = ora::State { graph->num_nodes };
			}
			if (results->cell_steps) results->cell_steps[i] = steps;
			if (results->items_needed) results->items_needed[i] = 0;
			if (results->traces_needed) results->traces_needed[i] = 0;
			uint32_t nt = 0;
			uint64_t used = 0;
			if (status == GA_OK)
			{
				uint64_t total = 0;
				for (const auto& t : traces) total += t.items.size();
				if (traces.size() > batch->max_traces || total > batch->trace_capacity[i])
				{
					status = GA_CAPACITY;
					if (results->items_needed) results->items_needed[i] = total;
					if (results->traces_needed) results->traces_needed[i] = (uint32_t)traces.size();
				}
				else
				{
					uint64_t* dst = results->trace_items + batch->trace_offset[i];
					for (const auto& t : traces)
					{
						const size_t k = (size_t)i * batch->max_traces + nt;
						results->trace_score[k] = t.score;
						results->trace_start[k] = used;
						results->trace_len[k] = (uint32_t)t.items.size();
						for (const auto& it : t.items) dst[used++] = packItem(it.node, it.nodeOffset, it.seqPos, it.nodeSwitch);
						nt++;
					}
				}
			}
			results->status[i] = status;
			results->num_traces[i] = nt;
		}
	};
	std::vector<std::thread> pool;
	for (int t = 1; t < threads; t++) pool.emplace_back(worker);
	worker();
	for (auto& t : pool) t.join();
	return GA_OK;
}
