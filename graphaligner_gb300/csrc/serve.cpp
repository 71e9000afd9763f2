// Serving loop over one resident graph and minimizer table: continuous batching of
// reads through seeding, the batched seed loop and GAF output (the request side of
// Aligner.cpp:440-592).
//
// One worker thread owns the requests.  Reads are served on lanes, each with its own
// seed-loop pool and extender, whose rounds run concurrently: reads of at least
// long_read_bp go to lane 0, the rest to the other lanes, so a short read never waits for
// a round that holds a long read's extensions.  Whenever a lane is idle the worker
//   1. admits queued reads of its class while the reads in flight stay under
//      max_reads_in_flight and their estimated band memory (read bp x band_bytes_per_bp)
//      under max_band_bytes -- a read that alone exceeds the budget is admitted when
//      nothing else is in flight;
//   2. seeds the admitted group (one k-mer lookup launch, host selection);
//   3. starts the lane's next round on a lane thread: the next seed's two extensions of
//      every read in the lane, old and new together, as one ga_extend_batch;
// and when a lane's round ends it finishes those seeds and publishes reads whose seed
// loop ended (selection + GAF) to the poll queue.  A read's seed loop only ever sees its
// own extensions' results and the extensions are independent DP runs, so its GAF bytes
// are the same whichever reads share its rounds or lane.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include "aligner.h"

void ga_set_last_error(const char* msg);

namespace
{
using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Submitted
{
    uint64_t ticket;
    std::string name;
    std::string seq;
    Clock::time_point submit;
};

struct Flight
{
    Clock::time_point submit;
    Clock::time_point admit;
    uint64_t bytes;
    uint64_t group;
    uint32_t lane;
};
}

struct ga_server
{
    ga_aligner* a = nullptr;
    uint32_t maxReads = 4096;
    uint64_t budget = 2ULL << 30;
    uint32_t bytesPerBp = 32;
    uint32_t lanes = 2;
    uint32_t longBp = 15000;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Submitted> queue[2];          // [0] long reads (lane 0), [1] the rest
    std::deque<ga_server_result> done;
    std::unordered_map<uint64_t, std::string> texts;
    uint64_t nextTicket = 1;
    bool stop = false;
    ga_server_stats stats {};
    std::thread worker;
    // the read class a lane serves
    int laneClass(uint32_t lane) const { return lanes > 1 && lane == 0 ? 0 : 1; }
    int readClass(size_t len) const { return lanes > 1 && len >= longBp ? 0 : 1; }
};

namespace
{
struct Lane
{
    std::unique_ptr<gahost::SeedLoopPool> pool;
    ExtendLane* ext = nullptr;
    std::unique_ptr<ExtendLane> owned;
    std::vector<gahost::ExtensionRequest> rq;
    std::vector<gahost::ExtensionResult> rs;
    std::thread thread;
    bool running = false;
    bool finished = false;                   // the round's thread is done (under ga_server::mu)
    std::map<uint64_t, size_t> groups;       // admission group -> reads of it in this lane
};
}

static void serve_loop(ga_server* s)
{
    ga_aligner* a = s->a;
    cudaSetDevice(a->device);
    // latency is the point here: one seed per read and round, no speculative seeds
    gahost::ReadAlignParams rp = ga_aligner_read_params(a);
    rp.maxSpeculation = 1;
    std::vector<Lane> lanes(s->lanes);
    for (uint32_t k = 0; k < s->lanes; k++)
    {
        lanes[k].pool.reset(new gahost::SeedLoopPool(*a->graph, rp));
        if (k == 0)
        {
            lanes[k].ext = &a->lanes[0];
            continue;
        }
        lanes[k].owned.reset(new ExtendLane());
        lanes[k].ext = lanes[k].owned.get();
        lanes[k].ext->params = &a->params.extend;
        if (ga_extender_create_like(a->ext, &lanes[k].ext->ext) != GA_OK)
        {
            // no device memory for another extender: serve every read on lane 0, including
            // long reads already queued for it
            std::lock_guard<std::mutex> lk(s->mu);
            s->lanes = 1;
            lanes.resize(1);
            for (auto& q : s->queue[0]) s->queue[1].push_back(std::move(q));
            s->queue[0].clear();
            break;
        }
        lanes[k].ext->owned = true;
    }
    gahost::BatchStats bs;
    std::vector<std::pair<uint64_t, gahost::ReadOutput>> fin;
    std::vector<std::pair<uint64_t, int32_t>> failedSeeding;
    std::unordered_map<uint64_t, Flight> flight;
    uint64_t inflightBytes = 0;
    uint64_t group = 0;

    auto publish = [&]()
    {
        if (fin.empty() && failedSeeding.empty()) return;
        const auto tDone = Clock::now();
        std::lock_guard<std::mutex> lk(s->mu);
        auto one = [&](uint64_t ticket, int32_t status, const gahost::ReadOutput* o)
        {
            auto f = flight.find(ticket);
            ga_server_result r {};
            r.ticket = ticket;
            r.status = status;
            std::string& text = s->texts[ticket];
            if (o)
            {
                text = o->gaf;
                r.alignments = (uint32_t)o->alignments;
                r.bp_aligned = o->bpAligned;
            }
            r.gaf = text.c_str();
            r.gaf_bytes = text.size();
            r.queue_ms = ms_between(f->second.submit, f->second.admit);
            r.latency_ms = ms_between(f->second.submit, tDone);
            inflightBytes -= f->second.bytes;
            auto& groups = lanes[f->second.lane].groups;
            auto g = groups.find(f->second.group);
            if (--g->second == 0) groups.erase(g);
            flight.erase(f);
            s->done.push_back(r);
            s->stats.completed++;
        };
        for (auto& fr : fin) one(fr.first, fr.second.failed ? GA_ASSERT : GA_OK, &fr.second);
        for (auto& fr : failedSeeding) one(fr.first, fr.second, nullptr);
        fin.clear();
        failedSeeding.clear();
        s->cvDone.notify_all();
    };

    while (true)
    {
        const auto t0 = Clock::now();
        bool worked = false;
        // rounds that ended: finish their seeds, publish finished reads
        for (auto& L : lanes)
        {
            bool ended;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                ended = L.running && L.finished;
            }
            if (!ended) continue;
            L.thread.join();
            L.running = false;
            L.pool->consume(L.rs, bs);
            L.pool->takeFinished(fin, bs);
            publish();
            worked = true;
        }
        // idle lanes: admit, seed, start the next round
        for (uint32_t k = 0; k < lanes.size(); k++)
        {
            Lane& L = lanes[k];
            if (L.running) continue;
            std::vector<Submitted> adm;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                auto& q = s->queue[s->laneClass(k)];
                while (!q.empty() && flight.size() + adm.size() < s->maxReads)
                {
                    const uint64_t b = (uint64_t)q.front().seq.size() * s->bytesPerBp;
                    if ((flight.size() + adm.size()) > 0 && inflightBytes + b > s->budget) break;
                    inflightBytes += b;
                    adm.push_back(std::move(q.front()));
                    q.pop_front();
                }
            }
            if (!adm.empty())
            {
                group++;
                const uint32_t n = (uint32_t)adm.size();
                std::vector<const char*> names(n);
                std::vector<uint64_t> offs(n);
                std::vector<uint32_t> lens(n);
                std::string blob;
                for (uint32_t i = 0; i < n; i++)
                {
                    names[i] = adm[i].name.c_str();
                    offs[i] = blob.size();
                    lens[i] = (uint32_t)adm[i].seq.size();
                    blob += adm[i].seq;
                }
                std::vector<gahost::ReadInput> reads;
                const int rc = ga_aligner_seed(a, n, names.data(), (const uint8_t*)blob.data(), offs.data(), lens.data(), reads);
                const auto now = Clock::now();
                std::vector<uint64_t> tags(n);
                for (uint32_t i = 0; i < n; i++)
                {
                    flight[adm[i].ticket] = Flight { adm[i].submit, now, (uint64_t)adm[i].seq.size() * s->bytesPerBp, group, k };
                    L.groups[group]++;
                    tags[i] = adm[i].ticket;
                    if (rc != GA_OK) failedSeeding.emplace_back(adm[i].ticket, rc);
                }
                if (rc == GA_OK) L.pool->addMany(reads, tags);
                std::lock_guard<std::mutex> lk(s->mu);
                s->stats.admissions++;
                s->stats.max_in_flight = std::max<uint64_t>(s->stats.max_in_flight, flight.size());
                worked = true;
            }
            const bool more = L.pool->collect(L.rq);
            L.pool->takeFinished(fin, bs);
            publish();
            if (!more) continue;
            worked = true;
            L.rs.assign(L.rq.size(), gahost::ExtensionResult {});
            {
                std::lock_guard<std::mutex> lk(s->mu);
                s->stats.rounds++;
                s->stats.extensions += L.rq.size();
                if (L.groups.size() > 1) s->stats.mixed_rounds++;
                L.finished = false;
            }
            L.running = true;
            L.thread = std::thread([s, &L]()
            {
                if (!L.rq.empty()) ga_aligner_extend(L.ext, L.rq, L.rs);
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    L.finished = true;
                }
                s->cvWork.notify_all();
            });
        }
        std::unique_lock<std::mutex> lk(s->mu);
        if (worked) s->stats.busy_ms += ms_between(t0, Clock::now());
        bool anyRunning = false;
        for (auto& L : lanes) anyRunning |= L.running;
        if (!anyRunning && flight.empty() && s->queue[0].empty() && s->queue[1].empty())
        {
            if (s->stop) break;
            s->cvWork.wait(lk, [&] { return s->stop || !s->queue[0].empty() || !s->queue[1].empty(); });
            continue;
        }
        if (worked) continue;
        // wait for a round to end or for work an idle lane can take
        s->cvWork.wait_for(lk, std::chrono::milliseconds(50), [&]
        {
            for (uint32_t k = 0; k < lanes.size(); k++)
            {
                if (lanes[k].running && lanes[k].finished) return true;
                if (!lanes[k].running && !s->queue[s->laneClass(k)].empty()) return true;
            }
            return s->stop;
        });
    }
}

extern "C" int ga_server_create(ga_aligner_t aligner, const ga_server_params* params, ga_server_t* out)
{
    if (!aligner || !out) return GA_ERR_ARGUMENT;
    if (aligner->params.multiseed_dp)
    {
        ga_set_last_error("ga_server_create: the serving loop runs the seed loop; the multiseed DP is ga_align_reads only");
        return GA_ERR_ARGUMENT;
    }
    ga_server* s = new ga_server();
    s->a = aligner;
    if (params)
    {
        if (params->max_reads_in_flight) s->maxReads = params->max_reads_in_flight;
        if (params->max_band_bytes) s->budget = params->max_band_bytes;
        if (params->band_bytes_per_bp) s->bytesPerBp = params->band_bytes_per_bp;
        if (params->lanes) s->lanes = std::min<uint32_t>(params->lanes, 8);
        if (params->long_read_bp) s->longBp = params->long_read_bp;
    }
    try
    {
        s->worker = std::thread(serve_loop, s);
    }
    catch (...)
    {
        delete s;
        ga_set_last_error("ga_server_create: cannot start the worker thread");
        return GA_ERR_ARGUMENT;
    }
    *out = s;
    return GA_OK;
}

extern "C" int ga_server_submit(ga_server_t s, const char* name, const uint8_t* seq, uint32_t len, uint64_t* ticket)
{
    if (!s || (len > 0 && !seq)) return GA_ERR_ARGUMENT;
    if (len > GA_MAX_SEQ_LEN)
    {
        ga_set_last_error("ga_server_submit: read longer than GA_MAX_SEQ_LEN (33,554,431 bp)");
        return GA_ERR_ARGUMENT;
    }
    Submitted q;
    q.name = name ? name : "";
    q.seq.assign((const char*)seq, len);
    q.submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return GA_ERR_ARGUMENT;
        q.ticket = s->nextTicket++;
        if (ticket) *ticket = q.ticket;
        s->queue[s->readClass(q.seq.size())].push_back(std::move(q));
        s->stats.submitted++;
    }
    s->cvWork.notify_one();
    return GA_OK;
}

extern "C" int ga_server_poll(ga_server_t s, ga_server_result* out, uint32_t max, uint32_t* count, int32_t wait_ms)
{
    if (!s || !count || (max > 0 && !out)) return GA_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] { return !s->done.empty(); };
    if (wait_ms < 0) s->cvDone.wait(lk, ready);
    else if (wait_ms > 0) s->cvDone.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
    uint32_t n = 0;
    while (n < max && !s->done.empty())
    {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *count = n;
    return GA_OK;
}

extern "C" int ga_server_release(ga_server_t s, uint64_t ticket)
{
    if (!s) return GA_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    s->texts.erase(ticket);
    return GA_OK;
}

extern "C" int ga_server_stats_get(ga_server_t s, ga_server_stats* out)
{
    if (!s || !out) return GA_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return GA_OK;
}

extern "C" int ga_server_free(ga_server_t s)
{
    if (!s) return GA_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cvWork.notify_all();
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return GA_OK;
}
