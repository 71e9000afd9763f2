// Test infrastructure only: a command-line driver around the REFERENCE's own
// hot-path source (GraphAligner src/), compiled by oracle/Makefile into
// oracle/_ref/ga_ref.  It produces the golden vectors the oracle restatement
// and the GPU kernels are checked against.  Nothing in the product links it.
//
// Modes
//   graphdump <graph.gfa> <out.gag>
//       Build the AlignmentGraph exactly as Aligner.cpp:getGraph does for GFA
//       (GfaGraph::LoadFromFile(.., true) + DirectedGraph::BuildFromGFA) and
//       write its device-visible arrays in the GAG1 layout the package reads.
//   extend <graph.gfa> <requests.tsv> <out.txt> <bandwidth> <Xdrop> <maxCells> <precise> [slices]
//       One GraphAlignerBitvectorBanded::getReverseTraceFromSeed call per
//       request line "bigraphNodeId offset sequence"
//       (GraphAlignerBitvectorBanded.h:59).  Writes status, score and every
//       trace item; with "slices" also dumps each DP slice's band.
//   align <graph.gfa> <reads.fa> <out.gaf> <preset vg|dbg> [bandwidth] [tangle] [multiseed]
//       One worker, in-order output: the GAF path of runComponentMappings
//       (Aligner.cpp:440-592) restated line by line with the reference calls;
//       "multiseed" takes the --multiseed-DP branch (PrepareMultiseeds,
//       AlignMultiseed, AddMappingQualities; Aligner.cpp:461-476).
//   seeds <graph.gfa> <reads.fa> <out.txt> <k> <w> <density> <discardFraction>
//       MinimizerSeeder::getSeeds + OrderSeeds per read.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <set>
#include <sstream>
#include <string>
#include <string_view>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#define private public
#include "AlignmentGraph.h"
#include "GfaGraph.h"
#include "BigraphToDigraph.h"
#include "GraphAlignerWrapper.h"
#include "GraphAligner.h"
// GraphAlignerBitvectorCommon.h defines a thread_local in the header, so the
// wrapper is compiled inside this translation unit rather than separately.
#include "GraphAlignerWrapper.cpp"
#include "MinimizerSeeder.h"
#include "AlignmentSelection.h"
#include "EValue.h"
#include "ThreadReadAssertion.h"
#undef private

using Common = GraphAlignerCommon<size_t, int32_t, uint64_t>;
using Banded = GraphAlignerBitvectorBanded<size_t, int32_t, uint64_t>;
using AlignerT = GraphAligner<size_t, int32_t, uint64_t>;

static AlignmentGraph loadGraph(const std::string& file)
{
	auto gfa = GfaGraph::LoadFromFile(file, true);
	return DirectedGraph::BuildFromGFA(gfa);
}

template <typename T>
static void writeVec(std::ofstream& out, const std::vector<T>& v)
{
	if (v.size() > 0) out.write((const char*)v.data(), v.size() * sizeof(T));
}

static void dumpGraph(const AlignmentGraph& g, const std::string& outFile)
{
	std::ofstream out { outFile, std::ios::binary };
	size_t N = g.nodeLength.size();
	std::vector<uint32_t> nodeLength(N), nodeOffset(N), component(N), inOff(N+1), outOff(N+1), inNb, outNb;
	std::vector<int32_t> nodeIDs(N);
	std::vector<uint8_t> reverse(N), linearizable(N);
	std::vector<uint64_t> chainNumber(N), chainApproxPos(N), seq2, seqAmb;
	for (size_t i = 0; i < N; i++)
	{
		nodeLength[i] = g.nodeLength[i];
		nodeOffset[i] = g.nodeOffset[i];
		component[i] = g.componentNumber[i];
		nodeIDs[i] = g.nodeIDs[i];
		reverse[i] = g.reverse[i];
		linearizable[i] = g.linearizable[i];
		chainNumber[i] = g.chainNumber[i];
		chainApproxPos[i] = g.chainApproxPos[i];
		inOff[i] = inNb.size();
		for (auto n : g.inNeighbors[i]) inNb.push_back(n);
		outOff[i] = outNb.size();
		for (auto n : g.outNeighbors[i]) outNb.push_back(n);
	}
	inOff[N] = inNb.size();
	outOff[N] = outNb.size();
	for (size_t i = 0; i < g.nodeSequences.size(); i++)
	{
		seq2.push_back(g.nodeSequences[i][0]);
		seq2.push_back(g.nodeSequences[i][1]);
	}
	for (size_t i = 0; i < g.ambiguousNodeSequences.size(); i++)
	{
		seqAmb.push_back(g.ambiguousNodeSequences[i].A);
		seqAmb.push_back(g.ambiguousNodeSequences[i].C);
		seqAmb.push_back(g.ambiguousNodeSequences[i].G);
		seqAmb.push_back(g.ambiguousNodeSequences[i].T);
	}
	std::vector<int32_t> lookupId;
	std::vector<uint32_t> originalSize, lookupOff, lookupIdx, nameLen;
	std::string names;
	for (const auto& pair : g.nodeLookup)
	{
		lookupId.push_back(pair.first);
		originalSize.push_back(g.originalNodeSize.at(pair.first));
		lookupOff.push_back(lookupIdx.size());
		for (auto n : pair.second) lookupIdx.push_back(n);
		std::string name = g.OriginalNodeName(pair.first);
		nameLen.push_back(name.size());
		names += name;
	}
	lookupOff.push_back(lookupIdx.size());
	out.write("GAG1", 4);
	uint64_t header[8] = { N, g.firstAmbiguous, inNb.size(), outNb.size(), lookupId.size(), lookupIdx.size(), names.size(), g.bpSize };
	out.write((const char*)header, sizeof(header));
	writeVec(out, nodeLength);
	writeVec(out, nodeIDs);
	writeVec(out, nodeOffset);
	writeVec(out, reverse);
	writeVec(out, linearizable);
	writeVec(out, component);
	writeVec(out, chainNumber);
	writeVec(out, chainApproxPos);
	writeVec(out, seq2);
	writeVec(out, seqAmb);
	writeVec(out, inOff);
	writeVec(out, inNb);
	writeVec(out, outOff);
	writeVec(out, outNb);
	writeVec(out, lookupId);
	writeVec(out, originalSize);
	writeVec(out, lookupOff);
	writeVec(out, lookupIdx);
	writeVec(out, nameLen);
	out.write(names.data(), names.size());
}

static void dumpSlices(std::ostream& out, const typename Banded::DPTable& table)
{
	for (size_t s = 0; s < table.slices.size(); s++)
	{
		const auto& sl = table.slices[s];
		out << "S " << (int64_t)sl.j << " " << sl.minScore << " " << (int64_t)sl.minScoreNode << " " << (int64_t)sl.minScoreNodeOffset << " " << sl.maxExactEndposScore << " " << (int64_t)sl.maxExactEndposNode << " " << sl.cellsProcessed << " " << (int)sl.scoresNotValid << " " << sl.bandwidth << " " << sl.scores.size();
		for (auto pair : sl.scores)
		{
			const auto& it = pair.second;
			out << " " << pair.first << ":" << it.startSlice.VP << "," << it.startSlice.VN << "," << it.startSlice.scoreEnd << "," << it.endSlice.VP << "," << it.endSlice.VN << "," << it.endSlice.scoreEnd << "," << it.HP[0] << "," << it.HN[0] << "," << it.minScore << "," << (int)it.exists;
		}
		out << "\n";
	}
}

static int runExtend(int argc, char** argv)
{
	if (argc < 9) { std::cerr << "extend <gfa> <requests> <out> <bw> <Xdrop> <maxCells> <precise> [slices]" << std::endl; return 1; }
	AlignmentGraph graph = loadGraph(argv[2]);
	size_t bandwidth = std::stoull(argv[5]);
	int Xdrop = std::stoi(argv[6]);
	size_t maxCells = std::stoull(argv[7]);
	double precise = std::stod(argv[8]);
	bool slices = argc > 9 && std::string(argv[9]) == "slices";
	Common::Params params { bandwidth, graph, maxCells, true, true, 1, 0, precise, Xdrop, 0 };
	Banded banded { params };
	Common::AlignerGraphsizedState state { graph, bandwidth };
	std::ifstream in { argv[3] };
	std::ofstream out { argv[4] };
	std::string line;
	size_t idx = 0;
	double totalSeconds = 0;
	while (std::getline(in, line))
	{
		if (line.size() == 0) continue;
		std::istringstream ls { line };
		int nodeId;
		size_t offset;
		std::string seq;
		ls >> nodeId >> offset >> seq;
		std::string_view view { seq.data(), seq.size() };
		int status = 0;
		Common::OnewayTrace trace;
		auto start = std::chrono::steady_clock::now();
		try
		{
			if (slices)
			{
				size_t numSlices = (view.size() + 63) / 64;
				auto init = GraphAlignerBitvectorCommon<size_t, int32_t, uint64_t>::getInitialSliceExactPosition(params, nodeId, offset);
				auto table = banded.getSlices(view, init, numSlices, Xdrop, state);
				dumpSlices(out, table);
			}
			trace = banded.getReverseTraceFromSeed(view, nodeId, offset, Xdrop, state);
		}
		catch (const ThreadReadAssertion::AssertionFailure&)
		{
			status = 2;
			state.clear();
		}
		totalSeconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
		if (status == 0 && trace.failed()) status = 1;
		out << "E " << idx << " " << status << " " << (status == 0 ? trace.score : 0) << " " << (status == 0 ? trace.trace.size() : 0);
		if (status == 0)
		{
			for (const auto& item : trace.trace)
			{
				out << " " << item.DPposition.node << "," << item.DPposition.nodeOffset << "," << (int64_t)item.DPposition.seqPos << "," << (int)item.nodeSwitch;
			}
		}
		out << "\n";
		idx++;
	}
	std::cerr << "extend: " << idx << " requests in " << totalSeconds << " s" << std::endl;
	return 0;
}

static std::vector<std::pair<std::string, std::string>> readFasta(const std::string& file)
{
	std::vector<std::pair<std::string, std::string>> result;
	std::ifstream in { file };
	std::string line;
	while (std::getline(in, line))
	{
		if (line.size() == 0) continue;
		if (line[0] == '>')
		{
			std::string name = line.substr(1);
			auto space = name.find_first_of(" \t");
			if (space != std::string::npos) name = name.substr(0, space);
			result.emplace_back(name, "");
		}
		else
		{
			result.back().second += line;
		}
	}
	return result;
}

struct Preset
{
	double minimizerSeedDensity = 0;
	size_t minimizerLength = 19;
	size_t minimizerWindowSize = 30;
	double seedExtendDensity = 0.002;
	size_t alignmentBandwidth = 0;
	size_t maxCellsPerSlice = std::numeric_limits<size_t>::max();
	double discard = 0.0002;
	double precise = 0.66;
	int Xdrop = 50;
	size_t clusterMin = 1;
	double multimapScoreFraction = 0.9;
	double minAlignmentScore = 0;
};

// AlignerMain.cpp:119-231 restated for the two presets plus -b / -C overrides.
static Preset makePreset(const std::string& name, int argc, char** argv, int firstExtra)
{
	Preset p;
	if (name == "dbg")
	{
		p.minimizerSeedDensity = 5; p.minimizerLength = 19; p.minimizerWindowSize = 30;
		p.seedExtendDensity = 0.002; p.alignmentBandwidth = 5; p.maxCellsPerSlice = 10000;
	}
	else if (name == "vg")
	{
		p.minimizerSeedDensity = 10; p.minimizerLength = 15; p.minimizerWindowSize = 20;
		p.seedExtendDensity = -1; p.discard = 0.001; p.alignmentBandwidth = 10;
	}
	if (argc > firstExtra && std::string(argv[firstExtra]) != "-") p.alignmentBandwidth = std::stoull(argv[firstExtra]);
	if (argc > firstExtra+1 && std::string(argv[firstExtra+1]) != "-") p.maxCellsPerSlice = std::stoull(argv[firstExtra+1]);
	if (p.precise >= 0.501) p.Xdrop = std::max((double)p.Xdrop, (double)50 * (100 * (p.precise / (1.0 - p.precise) + 1.0)));
	return p;
}

static int runAlign(int argc, char** argv)
{
	if (argc < 6) { std::cerr << "align <gfa> <reads.fa> <out.gaf> <preset> [bw] [tangle] [multiseed]" << std::endl; return 1; }
	AlignmentGraph graph = loadGraph(argv[2]);
	Preset p = makePreset(argv[5], argc, argv, 6);
	const bool multiseed = argc > 8 && std::string(argv[8]) == "multiseed";
	MinimizerSeeder seeder { graph, p.minimizerLength, p.minimizerWindowSize, 1, 1.0 - p.discard };
	auto reads = readFasta(argv[3]);
	std::ofstream out { argv[4] };
	Common::AlignerGraphsizedState reusableState { graph, p.alignmentBandwidth };
	AlignmentSelection::SelectionOptions selectionOptions;
	selectionOptions.graphSize = graph.SizeInBP();
	selectionOptions.ECutoff = -1;
	selectionOptions.minAlignmentScore = p.minAlignmentScore;
	selectionOptions.EValueCalc = EValueCalculator { p.precise };
	selectionOptions.AlignmentScoreFractionCutoff = p.multimapScoreFraction;
	size_t bpAlignedTotal = 0, failedAsserts = 0;
	auto wallStart = std::chrono::steady_clock::now();
	for (const auto& read : reads)
	{
		selectionOptions.readSize = read.second.size();
		AlignmentResult alignments;
		try
		{
			std::vector<SeedHit> seeds = seeder.getSeeds(read.second, p.minimizerSeedDensity);
			if (seeds.size() == 0) continue;
			if (multiseed)
			{
				PrepareMultiseeds(graph, seeds, read.second.size());
				alignments = AlignMultiseed(graph, read.first, read.second, p.alignmentBandwidth, p.maxCellsPerSlice, true, true, seeds, reusableState, p.clusterMin, p.seedExtendDensity, p.precise, p.Xdrop, p.multimapScoreFraction);
				AlignmentSelection::AddMappingQualities(alignments.alignments);
			}
			else
			{
				OrderSeeds(graph, seeds);
				alignments = AlignOneWay(graph, read.first, read.second, p.alignmentBandwidth, p.maxCellsPerSlice, true, true, seeds, reusableState, p.clusterMin, p.seedExtendDensity, p.precise, p.Xdrop);
			}
		}
		catch (const ThreadReadAssertion::AssertionFailure&)
		{
			reusableState.clear();
			failedAsserts++;
			continue;
		}
		if (alignments.alignments.size() > 0) alignments.alignments = AlignmentSelection::SelectAlignments(alignments.alignments, selectionOptions);
		if (alignments.alignments.size() == 0) continue;
		std::sort(alignments.alignments.begin(), alignments.alignments.end(), [](const AlignmentResult::AlignmentItem& left, const AlignmentResult::AlignmentItem& right) { return left.alignmentStart < right.alignmentStart; });
		size_t bpAligned = 0, lastEnd = 0;
		for (size_t i = 0; i < alignments.alignments.size(); i++)
		{
			size_t countStart = std::max(lastEnd, alignments.alignments[i].alignmentStart);
			if (alignments.alignments[i].alignmentEnd > countStart)
			{
				bpAligned += alignments.alignments[i].alignmentEnd - countStart;
				lastEnd = alignments.alignments[i].alignmentEnd;
			}
		}
		bpAlignedTotal += bpAligned;
		std::sort(alignments.alignments.begin(), alignments.alignments.end(), [](const AlignmentResult::AlignmentItem& left, const AlignmentResult::AlignmentItem& right) { return left.alignmentXScore > right.alignmentXScore; });
		try
		{
			for (size_t i = 0; i < alignments.alignments.size(); i++)
			{
				AddGAFLine(graph, read.first, read.second, alignments.alignments[i], false);
			}
		}
		catch (const ThreadReadAssertion::AssertionFailure&)
		{
			reusableState.clear();
			failedAsserts++;
			continue;
		}
		for (size_t i = 0; i < alignments.alignments.size(); i++)
		{
			out << alignments.alignments[i].GAFline << '\n';
		}
	}
	double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - wallStart).count();
	std::cerr << "align: reads " << reads.size() << " bpAligned " << bpAlignedTotal << " asserts " << failedAsserts << " seconds " << seconds << std::endl;
	return 0;
}

static int runSeeds(int argc, char** argv)
{
	if (argc < 9) { std::cerr << "seeds <gfa> <reads.fa> <out> <k> <w> <density> <discard>" << std::endl; return 1; }
	AlignmentGraph graph = loadGraph(argv[2]);
	size_t k = std::stoull(argv[5]);
	size_t w = std::stoull(argv[6]);
	double density = std::stod(argv[7]);
	double discard = std::stod(argv[8]);
	MinimizerSeeder seeder { graph, k, w, 1, 1.0 - discard };
	auto reads = readFasta(argv[3]);
	std::ofstream out { argv[4] };
	out << "maxCount " << seeder.maxCount << "\n";
	for (const auto& read : reads)
	{
		auto seeds = seeder.getSeeds(read.second, density);
		out << "R " << read.first << " " << seeds.size();
		for (const auto& s : seeds) out << " " << s.nodeID << "," << s.nodeOffset << "," << s.seqPos << "," << s.matchLen << "," << s.reverse << "," << s.alignmentGraphNodeId << "," << s.alignmentGraphNodeOffset << "," << s.rawSeedGoodness;
		out << "\n";
		OrderSeeds(graph, seeds);
		out << "O " << read.first << " " << seeds.size();
		for (const auto& s : seeds) out << " " << s.nodeID << "," << s.nodeOffset << "," << s.seqPos << "," << s.seedGoodness << "," << s.seedClusterSize;
		out << "\n";
	}
	return 0;
}

int main(int argc, char** argv)
{
	if (argc < 2) { std::cerr << "modes: graphdump extend align seeds" << std::endl; return 1; }
	std::string mode = argv[1];
	if (mode == "graphdump")
	{
		if (argc < 4) return 1;
		AlignmentGraph graph = loadGraph(argv[2]);
		dumpGraph(graph, argv[3]);
		return 0;
	}
	if (mode == "extend") return runExtend(argc, argv);
	if (mode == "align") return runAlign(argc, argv);
	if (mode == "seeds") return runSeeds(argc, argv);
	std::cerr << "unknown mode " << mode << std::endl;
	return 1;
}
