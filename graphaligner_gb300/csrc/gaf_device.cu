// GAF lines and alignment selection on the GPU (GraphAlignerGAFAlignment::traceToAlignment,
// GraphAlignerGAFAlignment.h:37-200; AlignmentSelection::SelectAlignments,
// AlignmentSelection.cpp:31-95).
//
// The host's cores walk each selected alignment's trace once (gaf::classify_line: one edit-op
// byte per trace item, the node-path entries, the counts), between seed-loop rounds; the ops,
// entries and line records go down in chunks, one thread per line measures its line, the host
// places the lines, and one thread per line writes it (names, numbers, the doubles, the
// CIGAR's runs).  The node names,
// the bigraph-id lookup and the node sizes stay resident from the aligner's creation.
// Selection runs one thread per read over its alignments' spans and X-scores.
#include <cuda_runtime.h>
#include <chrono>
#include <cmath>
#include <cstring>
#include "aligner.h"
#include "extend.cuh"

namespace
{

__global__ void gaf_measure_kernel(gaf::Names nm, const gaf::LineMeta* lines, const uint8_t* ops, const int32_t* entries, uint32_t n, int64_t* len)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) len[k] = gaf::write_line(nm, lines[k], ops, entries, nullptr);
}

__global__ void gaf_write_kernel(gaf::Names nm, const gaf::LineMeta* lines, const uint8_t* ops, const int32_t* entries, uint32_t n,
    const uint64_t* start, char* text)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    char* out = text + start[k];
    const int64_t len = gaf::write_line(nm, lines[k], ops, entries, out);
    out[len] = '\n';
}

__global__ void select_kernel(const uint64_t* first, const uint64_t* start, const uint64_t* end, const double* score, uint32_t n,
    int minAlignmentScore, double fraction, char* keep)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t a = first[r];
    gaf::select_read((uint32_t)(first[r + 1] - a), start + a, end + a, score + a, minAlignmentScore, fraction, keep + a);
}

double ms_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

gaf::Names device_names(const GafDevice& d)
{
    gaf::Names nm {};
    nm.nodeNames = d.nodeNames.p;
    nm.nodeNameOff = d.nodeNameOff.p;
    nm.originalSize = d.originalSize.p;
    nm.idKey = d.idKey.p;
    nm.idVal = d.idVal.p;
    nm.idCap = d.idCap;
    return nm;
}

template <typename T>
bool upload(DevGrow<T>& dst, const std::vector<T>& src, cudaStream_t s)
{
    return dst.reserve(std::max<size_t>(src.size(), 1))
        && (src.empty() || cudaMemcpyAsync(dst.p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s) == cudaSuccess);
}

// edit ops of at most this many trace items go down at once
constexpr uint64_t kChunkOps = 1ULL << 27;

// Writes the classified lines of reads on the device in chunks and appends them, each with its
// newline, to text; readEnd[i] = where read i's text ends.  False on a CUDA error.
bool write_reads(GafDevice& d, const std::vector<const std::string*>& names, const std::vector<const gahost::ClassifiedLines*>& reads,
    std::string& text, std::vector<uint64_t>& readEnd)
{
    const size_t n = reads.size();
    text.clear();
    readEnd.assign(n, 0);
    cudaStream_t s = d.stream;
    size_t from = 0;
    while (from < n)
    {
        size_t to = from;
        uint64_t ops = 0;
        while (to < n && (to == from || ops + reads[to]->ops.size() <= kChunkOps)) ops += reads[to++]->ops.size();
        const size_t m = to - from;
        // where each read's lines, ops, entries and name go in the chunk
        std::vector<uint64_t> lineAt(m + 1, 0), opAt(m + 1, 0), entryAt(m + 1, 0);
        uint64_t nameBytes = 0;
        for (size_t k = 0; k < m; k++)
        {
            const auto& c = *reads[from + k];
            lineAt[k + 1] = lineAt[k] + c.lines.size();
            opAt[k + 1] = opAt[k] + c.ops.size();
            entryAt[k + 1] = entryAt[k] + c.entries.size();
            nameBytes += names[from + k]->size();
        }
        const uint64_t lines = lineAt[m], entries = entryAt[m];
        if (!d.hOps.reserve(std::max<uint64_t>(ops, 1)) || !d.hMeta.reserve(std::max<uint64_t>(lines, 1)) || !d.hEntries.reserve(std::max<uint64_t>(entries, 1))
            || !d.hNames.reserve(std::max<uint64_t>(nameBytes, 1)) || !d.hNameOff.reserve(m + 1) || !d.hLen.reserve(std::max<uint64_t>(lines, 1))
            || !d.hStart.reserve(std::max<uint64_t>(lines, 1)))
            return false;
        uint64_t at = 0;
        for (size_t k = 0; k < m; k++)
        {
            d.hNameOff[k] = at;
            at += names[from + k]->size();
        }
        d.hNameOff[m] = at;
        gahost::parallelFor(m, [&](size_t k)
        {
            const auto& c = *reads[from + k];
            memcpy(d.hNames.p + d.hNameOff[k], names[from + k]->data(), names[from + k]->size());
            if (!c.ops.empty()) memcpy(d.hOps.p + opAt[k], c.ops.data(), c.ops.size());
            if (!c.entries.empty()) memcpy(d.hEntries.p + entryAt[k], c.entries.data(), c.entries.size() * 4);
            for (size_t q = 0; q < c.lines.size(); q++)
            {
                gaf::LineMeta meta = c.lines[q];
                meta.op += opAt[k];
                meta.entry += entryAt[k];
                meta.read = (uint32_t)k;
                d.hMeta[lineAt[k] + q] = meta;
            }
        });
        if (!d.ops.reserve(std::max<uint64_t>(ops, 1)) || !d.meta.reserve(std::max<uint64_t>(lines, 1)) || !d.entries.reserve(std::max<uint64_t>(entries, 1))
            || !d.names.reserve(std::max<uint64_t>(nameBytes, 1)) || !d.nameOff.reserve(m + 1) || !d.len.reserve(std::max<uint64_t>(lines, 1))
            || !d.start.reserve(std::max<uint64_t>(lines, 1)))
            return false;
        if ((ops && cudaMemcpyAsync(d.ops.p, d.hOps.p, ops, cudaMemcpyHostToDevice, s) != cudaSuccess)
            || (lines && cudaMemcpyAsync(d.meta.p, d.hMeta.p, lines * sizeof(gaf::LineMeta), cudaMemcpyHostToDevice, s) != cudaSuccess)
            || (entries && cudaMemcpyAsync(d.entries.p, d.hEntries.p, entries * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
            || (nameBytes && cudaMemcpyAsync(d.names.p, d.hNames.p, nameBytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
            || cudaMemcpyAsync(d.nameOff.p, d.hNameOff.p, (m + 1) * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return false;
        gaf::Names nm = device_names(d);
        nm.readNames = d.names.p;
        nm.readNameOff = d.nameOff.p;
        nm.readLen = nullptr;
        const uint32_t blocks = (uint32_t)((lines + 127) / 128);
        if (lines)
        {
            gaf_measure_kernel<<<blocks, 128, 0, s>>>(nm, d.meta.p, d.ops.p, d.entries.p, (uint32_t)lines, d.len.p);
            if (cudaGetLastError() != cudaSuccess) return false;
            if (cudaMemcpyAsync(d.hLen.p, d.len.p, lines * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
                return false;
        }
        uint64_t total = 0;
        const uint64_t base = text.size();
        for (size_t k = 0; k < m; k++)
        {
            for (uint64_t q = lineAt[k]; q < lineAt[k + 1]; q++)
            {
                d.hStart[q] = total;
                total += (uint64_t)d.hLen[q] + 1;
            }
            readEnd[from + k] = base + total;
        }
        if (lines)
        {
            if (!d.text.reserve(std::max<uint64_t>(total, 1))) return false;
            if (cudaMemcpyAsync(d.start.p, d.hStart.p, lines * 8, cudaMemcpyHostToDevice, s) != cudaSuccess) return false;
            gaf_write_kernel<<<blocks, 128, 0, s>>>(nm, d.meta.p, d.ops.p, d.entries.p, (uint32_t)lines, d.start.p, d.text.p);
            if (cudaGetLastError() != cudaSuccess) return false;
            text.resize(base + total);
            if (cudaMemcpyAsync(&text[base], d.text.p, total, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
                return false;
        }
        from = to;
    }
    return true;
}

}

int ga_gaf_device_init(GafDevice& d, const gahost::HostGraph& g)
{
    cudaGetDevice(&d.device);
    if (!d.stream && cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking) != cudaSuccess) return GA_ERR_CUDA;
    gaf::build_names(g.lookupIds, g.names, g.originalSize, d.host);
    cudaStream_t s = d.stream;
    if (!upload(d.nodeNames, d.host.nodeNames, s) || !upload(d.nodeNameOff, d.host.nodeNameOff, s) || !upload(d.originalSize, d.host.originalSize, s)
        || !upload(d.idKey, d.host.idKey, s) || !upload(d.idVal, d.host.idVal, s) || cudaStreamSynchronize(s) != cudaSuccess)
        return GA_ERR_CUDA;
    d.idCap = d.host.idCap;
    return GA_OK;
}

bool ga_gaf_device_write(void* ctx, const std::vector<const std::string*>& names, const std::vector<const gahost::ClassifiedLines*>& reads,
    std::string& text, std::vector<uint64_t>& readEnd)
{
    GafDevice& d = *(GafDevice*)ctx;
    const auto t0 = std::chrono::steady_clock::now();
    const bool ok = write_reads(d, names, reads, text, readEnd);
    if (!ok) ga_set_last_error("GAF lines on the device failed");
    d.ms += ms_since(t0);
    return ok;
}

bool ga_gaf_device_select(void* ctx, const std::vector<uint64_t>& first, const std::vector<uint64_t>& start, const std::vector<uint64_t>& end,
    const std::vector<double>& xscore, int minAlignmentScore, double fractionCutoff, std::vector<char>& keep)
{
    GafDevice& d = *(GafDevice*)ctx;
    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t reads = (uint32_t)(first.size() - 1);
    const uint64_t m = start.size();
    cudaStream_t s = d.stream;
    bool ok = d.hSel.reserve(first.size() + 2 * m) && d.hScore.reserve(std::max<uint64_t>(m, 1)) && d.hKeep.reserve(std::max<uint64_t>(m, 1))
        && d.sel.reserve(first.size() + 2 * m) && d.score.reserve(std::max<uint64_t>(m, 1)) && d.keep.reserve(std::max<uint64_t>(m, 1));
    if (ok)
    {
        memcpy(d.hSel.p, first.data(), first.size() * 8);
        memcpy(d.hSel.p + first.size(), start.data(), m * 8);
        memcpy(d.hSel.p + first.size() + m, end.data(), m * 8);
        memcpy(d.hScore.p, xscore.data(), m * 8);
        ok = cudaMemcpyAsync(d.sel.p, d.hSel.p, (first.size() + 2 * m) * 8, cudaMemcpyHostToDevice, s) == cudaSuccess
            && cudaMemcpyAsync(d.score.p, d.hScore.p, m * 8, cudaMemcpyHostToDevice, s) == cudaSuccess;
    }
    if (ok)
    {
        select_kernel<<<(reads + 127) / 128, 128, 0, s>>>(d.sel.p, d.sel.p + first.size(), d.sel.p + first.size() + m, d.score.p, reads,
            minAlignmentScore, fractionCutoff, d.keep.p);
        ok = cudaGetLastError() == cudaSuccess && cudaMemcpyAsync(d.hKeep.p, d.keep.p, m, cudaMemcpyDeviceToHost, s) == cudaSuccess
            && cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (ok) memcpy(keep.data(), d.hKeep.p, m);
    else ga_set_last_error("alignment selection on the device failed");
    d.ms += ms_since(t0);
    return ok;
}

// ---- C ABI ----

extern "C" int ga_aligner_format_gaf(ga_aligner_t a, uint32_t num_lines, const ga_gaf_line* lines, uint64_t num_items, const ga_gaf_item* items,
    uint32_t num_reads, const char* const* read_names, const uint32_t* read_lens, uint8_t cigar_match_mismatch, const char** text, uint64_t* bytes,
    const uint64_t** line_ends, const uint8_t** failed)
{
    static_assert(sizeof(ga_gaf_item) == sizeof(gaf::Item) && sizeof(ga_gaf_line) == sizeof(gaf::Line), "GAF record layouts");
    if (!a || !text || !bytes || !line_ends || !failed || (num_lines && !lines) || (num_items && !items) || (num_reads && (!read_names || !read_lens)))
        return GA_ERR_ARGUMENT;
    GafDevice& d = a->gafDev;
    for (uint32_t k = 0; k < num_lines; k++)
    {
        const ga_gaf_line& l = lines[k];
        if (l.read >= num_reads || l.first_item + l.item_count > num_items || l.item_count == 0)
        {
            ga_set_last_error(("ga_aligner_format_gaf: line " + std::to_string(k) + " names a read or items it was not given").c_str());
            return GA_ERR_ARGUMENT;
        }
    }
    // each line is walked on the host's cores, then the good ones are written on the device
    const gaf::NamesHost& nh = d.host;
    auto sizeOf = [&nh](int32_t bignode) -> uint64_t
    {
        uint64_t h = gaf::id_hash(bignode) & (nh.idCap - 1);
        for (uint64_t k = 0; k < nh.idCap; k++)
        {
            if (nh.idKey[h] == bignode) return nh.originalSize[nh.idVal[h]];
            if (nh.idKey[h] == INT32_MIN) return 0;
            h = (h + 1) & (nh.idCap - 1);
        }
        return 0;
    };
    std::vector<gahost::ClassifiedLines> cls(num_lines);
    std::vector<std::string> names(num_lines);
    d.lastFailed.assign(num_lines, 0);
    gahost::parallelFor(num_lines, [&](size_t k)
    {
        const ga_gaf_line& l = lines[k];
        const gaf::Item* it = (const gaf::Item*)items + l.first_item;
        gahost::ClassifiedLines& c = cls[k];
        c.lines.resize(1);
        c.ops.resize(l.item_count);
        c.entries.resize(l.item_count);
        gaf::LineMeta& m = c.lines[0];
        if (!gaf::classify_line([it](uint32_t q) { return it[q]; }, l.item_count, read_lens[l.read], cigar_match_mismatch != 0, sizeOf, m,
                c.ops.data(), c.entries.data()))
        {
            d.lastFailed[k] = 1;
            c = gahost::ClassifiedLines {};
            return;
        }
        m.op = 0;
        m.entry = 0;
        m.xscore100 = l.xscore100;
        m.mapq = l.mapq;
        c.entries.resize(m.entries);
        names[k] = read_names[l.read] ? read_names[l.read] : "";
    });
    std::vector<const std::string*> np;
    std::vector<const gahost::ClassifiedLines*> rp;
    for (uint32_t k = 0; k < num_lines; k++)
    {
        if (d.lastFailed[k]) continue;
        np.push_back(&names[k]);
        rp.push_back(&cls[k]);
    }
    std::string body;
    std::vector<uint64_t> ends;
    if (!write_reads(d, np, rp, body, ends))
    {
        ga_set_last_error("ga_aligner_format_gaf: device formatting failed");
        return GA_ERR_CUDA;
    }
    // the text in line order, a failed line as a lone newline
    d.lastText.clear();
    d.lastEnds.assign(num_lines, 0);
    size_t g = 0;
    uint64_t prev = 0;
    for (uint32_t k = 0; k < num_lines; k++)
    {
        if (d.lastFailed[k]) d.lastText += '\n';
        else
        {
            d.lastText.append(body, prev, ends[g] - prev);
            prev = ends[g++];
        }
        d.lastEnds[k] = d.lastText.size();
    }
    *text = d.lastText.data();
    *bytes = d.lastText.size();
    *line_ends = d.lastEnds.data();
    *failed = d.lastFailed.data();
    return GA_OK;
}

extern "C" int ga_aligner_select_alignments(ga_aligner_t a, uint32_t num_reads, const uint64_t* first, const uint64_t* starts,
    const uint64_t* ends, const double* xscores, int32_t min_alignment_score, double multimap_score_fraction, uint8_t* keep)
{
    if (!a || !first || !keep || (num_reads && (!starts || !ends || !xscores))) return GA_ERR_ARGUMENT;
    std::vector<uint64_t> f(first, first + num_reads + 1);
    for (uint32_t r = 0; r < num_reads; r++)
        if (f[r + 1] < f[r]) return GA_ERR_ARGUMENT;
    const uint64_t m = f[num_reads] - f[0];
    for (auto& x : f) x -= first[0];
    std::vector<uint64_t> s(starts + first[0], starts + first[0] + m), e(ends + first[0], ends + first[0] + m);
    std::vector<double> x(xscores + first[0], xscores + first[0] + m);
    std::vector<char> k(m, 0);
    if (m && !ga_gaf_device_select(&a->gafDev, f, s, e, x, min_alignment_score, multimap_score_fraction, k)) return GA_ERR_CUDA;
    for (uint64_t i = 0; i < m; i++) keep[first[0] + i] = (uint8_t)k[i];
    return GA_OK;
}
