// Test-infrastructure shim (oracle build only): the reference generates vg.pb.h
// from src/vg.proto with protoc, which is not available here.  These plain
// structs expose the accessor/mutator names the reference's host code calls
// (BigraphToDigraph.cpp, CommonUtils.cpp, GraphAlignerVGAlignment.h) so that
// the GFA path compiles.  GAM/JSON output is not exercised by the oracle.
#pragma once
#include <string>
#include <vector>
#include <deque>
#include <cstdint>

namespace vg
{

#define VGSHIM_FIELD(type, name) \
	type name##_ {}; \
	const type& name() const { return name##_; } \
	void set_##name(const type& v) { name##_ = v; }

class Position
{
public:
	VGSHIM_FIELD(int64_t, node_id)
	VGSHIM_FIELD(int64_t, offset)
	VGSHIM_FIELD(bool, is_reverse)
	VGSHIM_FIELD(std::string, name)
};

class Edit
{
public:
	VGSHIM_FIELD(int32_t, from_length)
	VGSHIM_FIELD(int32_t, to_length)
	VGSHIM_FIELD(std::string, sequence)
};

class Mapping
{
public:
	Position* mutable_position() { return &position_; }
	const Position& position() const { return position_; }
	void set_allocated_position(Position* p) { position_ = *p; delete p; }
	Edit* add_edit() { edits.emplace_back(); return &edits.back(); }
	int edit_size() const { return (int)edits.size(); }
	const Edit& edit(int i) const { return edits[i]; }
	VGSHIM_FIELD(int64_t, rank)
private:
	Position position_;
	std::deque<Edit> edits;
};

class Path
{
public:
	Mapping* add_mapping() { mappings.emplace_back(); return &mappings.back(); }
	Mapping* mutable_mapping(int i) { return &mappings[i]; }
	const Mapping& mapping(int i) const { return mappings[i]; }
	int mapping_size() const { return (int)mappings.size(); }
	VGSHIM_FIELD(std::string, name)
private:
	std::deque<Mapping> mappings;
};

class Alignment
{
public:
	Path* mutable_path() { return &path_; }
	const Path& path() const { return path_; }
	void set_allocated_path(Path* p) { path_ = *p; delete p; }
	VGSHIM_FIELD(std::string, name)
	VGSHIM_FIELD(std::string, sequence)
	VGSHIM_FIELD(int32_t, score)
	VGSHIM_FIELD(double, identity)
	VGSHIM_FIELD(int64_t, query_position)
	VGSHIM_FIELD(int32_t, mapping_quality)
	bool SerializeToString(std::string*) const { return false; }
	bool ParseFromString(const std::string&) { return false; }
private:
	Path path_;
};

class Node
{
public:
	VGSHIM_FIELD(int64_t, id)
	VGSHIM_FIELD(std::string, sequence)
	VGSHIM_FIELD(std::string, name)
};

class Edge
{
public:
	VGSHIM_FIELD(int64_t, from)
	VGSHIM_FIELD(int64_t, to)
	VGSHIM_FIELD(bool, from_start)
	VGSHIM_FIELD(bool, to_end)
	VGSHIM_FIELD(int32_t, overlap)
};

class Graph
{
public:
	Node* add_node() { nodes.emplace_back(); return &nodes.back(); }
	Edge* add_edge() { edges.emplace_back(); return &edges.back(); }
	int node_size() const { return (int)nodes.size(); }
	int edge_size() const { return (int)edges.size(); }
	const Node& node(int i) const { return nodes[i]; }
	const Edge& edge(int i) const { return edges[i]; }
	bool SerializeToString(std::string*) const { return false; }
	bool ParseFromString(const std::string&) { return false; }
private:
	std::deque<Node> nodes;
	std::deque<Edge> edges;
};

#undef VGSHIM_FIELD

}
