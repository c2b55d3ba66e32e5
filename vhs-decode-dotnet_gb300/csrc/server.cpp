// Window server: the serving loop of the decode path.
//
// Clients submit decode windows (RF sample ranges of one client stream, any
// supported format) as they arrive; worker threads decode them concurrently,
// each on its own device slot (a session with its own streams), so windows
// that arrive while others are on the GPU are admitted as soon as a worker
// and device memory are free and their kernels overlap on the device.
//
// Slots are created on demand for a (profile, tape speed, tape format, sample
// rate, decimation) and
// kept; a new slot is admitted only while the device-memory footprint of all
// slots stays inside the server's budget, otherwise an idle slot of another
// format is released or the window waits in the queue.  Windows of one
// client stream are decoded in submission order, and the stream's sync
// history (field parity, hsync history, continuation point of the next
// field) carries from one window to the next unless the window is marked as
// a seek.  This replaces the reference's single-window preview context
// (src/VHSDecode.CudaFast.Native/include/vhsdecode_cuda_fast.h:158-171), which
// decodes one window at a time behind a mutex.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "session.hpp"

using namespace vhsd;
using namespace vhsd::detail;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Slot {
    vhsdecode_gb300_session* s = nullptr;
    uint32_t profile = 0, speed = 0, tape_format = 0, decim = 1;
    double mhz = 0.0;
    size_t bytes = 0;
    bool busy = false;
    Clock::time_point last_used;
};

struct Request {
    uint64_t ticket = 0;
    vhsdecode_gb300_window_v1 w{};
    Clock::time_point submitted;
};

struct History {
    bool valid = false;
    FieldState state;
    uint64_t next_abs = 0;  // source-sample position of the next field span (stream coordinates)
    int64_t vhs_abs = 0;    // source-sample position of the last field's read location
    bool busy = false;
};

}  // namespace

struct vhsdecode_gb300_server {
    vhsdecode_gb300_server_config_v1 cfg{};
    size_t budget = 0, used = 0;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::map<uint64_t, vhsdecode_gb300_window_result_v1> done;
    std::unordered_map<uint32_t, History> streams;
    std::vector<Slot*> slots;
    std::vector<std::thread> workers;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::mutex create_m;   // slot creations one at a time, so their footprints measure cleanly
};

namespace {

uint32_t window_decim(const vhsdecode_gb300_window_v1& w) { return w.decimation == 2 ? 2u : 1u; }

bool same_format(const Slot& sl, const vhsdecode_gb300_window_v1& w) {
    return sl.profile == w.profile && sl.speed == w.tape_speed && sl.tape_format == w.tape_format &&
           sl.mhz == w.sample_rate_mhz && sl.decim == window_decim(w);
}

// Device footprint of one slot, measured when the first slot of a format is
// made; an estimate (bytes per capacity sample plus fixed tables) before that.
size_t estimate_slot_bytes(const vhsdecode_gb300_server* sv) {
    return (size_t)(16.5 * (double)sv->cfg.max_window_samples) + ((size_t)256 << 20);
}

// Picks the first queued window whose stream is idle and for which a slot can
// be had: an idle slot of its format, a new slot inside the budget, or a new
// slot after releasing idle slots of other formats.  Returns false if none.
bool pick(vhsdecode_gb300_server* sv, Request& out, Slot*& slot, std::vector<Slot*>& release,
          bool batch_only = false) {
    for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it) {
        History& h = sv->streams[it->w.stream_id];
        if (h.busy) continue;
        if (batch_only && window_decim(it->w) != 1) continue;   // decimated windows decode alone
        Slot* found = nullptr;
        for (Slot* sl : sv->slots)
            if (!sl->busy && same_format(*sl, it->w)) { found = sl; break; }
        if (!found) {
            // footprint: measured on a slot of this format, else the largest
            // measured slot, else the estimate; the first slot is always admitted
            size_t need = 0;
            for (Slot* sl : sv->slots)
                if (same_format(*sl, it->w)) { need = sl->bytes; break; }
            if (!need)
                for (Slot* sl : sv->slots) need = std::max(need, sl->bytes);
            if (!need) need = estimate_slot_bytes(sv);
            if (sv->slots.empty()) need = std::min(need, sv->budget);
            size_t freeable = 0;
            std::vector<Slot*> idle_other;
            for (Slot* sl : sv->slots)
                if (!sl->busy && !same_format(*sl, it->w)) { idle_other.push_back(sl); freeable += sl->bytes; }
            if (sv->used + need > sv->budget) {
                if (sv->used - freeable + need > sv->budget) continue;  // wait for memory
                // release least recently used idle slots of other formats until it fits
                std::sort(idle_other.begin(), idle_other.end(),
                          [](const Slot* a, const Slot* b) { return a->last_used < b->last_used; });
                size_t used = sv->used;
                for (Slot* sl : idle_other) {
                    if (used + need <= sv->budget) break;
                    used -= sl->bytes;
                    release.push_back(sl);
                }
            }
            for (Slot* sl : release) {
                sv->slots.erase(std::find(sv->slots.begin(), sv->slots.end(), sl));
                sv->used -= sl->bytes;
            }
            found = new Slot;
            found->profile = it->w.profile;
            found->speed = it->w.tape_speed;
            found->tape_format = it->w.tape_format;
            found->mhz = it->w.sample_rate_mhz;
            found->decim = window_decim(it->w);
            found->bytes = need;   // reserved now, corrected after creation
            sv->used += need;
            sv->slots.push_back(found);
        }
        found->busy = true;
        h.busy = true;
        out = *it;
        sv->queue.erase(it);
        slot = found;
        return true;
    }
    return false;
}

void create_slot(vhsdecode_gb300_server* sv, Slot* sl) {
    vhsdecode_gb300_session_config_v1 c{};
    c.struct_size = sizeof(c);
    c.profile = sl->profile;
    c.tape_speed = sl->speed;
    c.tape_format = sl->tape_format;
    c.device_id = sv->cfg.device_id;
    c.sample_rate_mhz = sl->mhz;
    c.max_samples = sv->cfg.max_window_samples;
    c.precision = VHSDECODE_GB300_PRECISION_FP32_FUSED;
    c.decimation = sl->decim;
    size_t f0 = 0, f1 = 0, total = 0;
    std::lock_guard<std::mutex> create_lock(sv->create_m);
    ck(cudaSetDevice(sv->cfg.device_id), "cudaSetDevice");
    cudaMemGetInfo(&f0, &total);
    auto* s = new vhsdecode_gb300_session();
    try {
        session_init(s, c);
    } catch (...) {
        session_free(s);
        delete s;
        throw;
    }
    cudaMemGetInfo(&f1, &total);
    sl->s = s;
    if (f0 > f1) {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->used = sv->used - sl->bytes + (f0 - f1);
        sl->bytes = f0 - f1;
    }
}

void destroy_slot(Slot* sl) {
    if (sl->s) {
        cudaStreamSynchronize(sl->s->stream);
        session_free(sl->s);
        delete sl->s;
    }
    delete sl;
}

// The decode carry of a window: a window that continues its stream (no seek,
// starting at or before the stream's next field) resumes the stream's field
// sequence at that field.
bool window_carry(const vhsdecode_gb300_window_v1& w, const History& hist, DecodeCarry& carry) {
    const uint64_t decim = window_decim(w);
    carry = DecodeCarry{};
    carry.no_graph = true;   // every window has its own input pointer
    const bool cont = !w.seek && hist.valid && hist.next_abs >= w.source_offset;
    if (cont) {
        carry.state = hist.state;
        carry.state.vhs_loc = (hist.vhs_abs - (int64_t)w.source_offset) / (int64_t)decim;
        carry.start = (int64_t)((hist.next_abs - w.source_offset) / decim);
    }
    return cont;
}

// Results of a decoded window: its TBC to the client's buffer, the window
// result and the stream's history after it.
void window_finish(vhsdecode_gb300_session* s, const vhsdecode_gb300_window_v1& w, const DecodeCarry& carry,
                   bool cont, const vhsdecode_gb300_decode_result_v1& dr, vhsdecode_gb300_window_result_v1& r,
                   History& out_hist) {
    const uint64_t decim = window_decim(w);
    size_t per_field = (size_t)s->out_lines * s->outlen;
    if (w.tbc_out && dr.fields) {
        size_t nf = std::min<size_t>(dr.fields, w.tbc_capacity / per_field);
        if (nf) ck(cudaMemcpyAsync(w.tbc_out, s->tbc.p, nf * per_field * sizeof(uint16_t), cudaMemcpyDeviceToHost,
                                   s->stream), "d2h tbc");
        ck(cudaStreamSynchronize(s->stream), "sync");
    }
    r.fields = dr.fields;
    r.first_field_is_first = (dr.fields && s->fields[0].sync.first_field) ? 1u : 0u;
    r.continued = cont ? 1u : 0u;
    // A window that starts on the stream's block and span grid (multiples of
    // lcm(30720, 32768) = 983040 decoded samples from where the stream began)
    // decodes its fields exactly as one decode of the whole stream would
    // (decimated windows: up to the decimator's zero taps before the window).
    const int64_t grid = 983040;
    int64_t back = std::max<int64_t>(0, carry.next - 2 * kBlock);
    r.next_source_offset = w.source_offset + decim * (uint64_t)((back / grid) * grid);
    out_hist.valid = dr.fields > 0;
    out_hist.state = carry.state;
    out_hist.next_abs = w.source_offset + decim * (uint64_t)std::max<int64_t>(0, carry.next);
    out_hist.vhs_abs = (int64_t)w.source_offset + (int64_t)decim * carry.state.vhs_loc;
}

void run_window(Slot* sl, const Request& rq, const History& hist, vhsdecode_gb300_window_result_v1& r,
                History& out_hist) {
    DecodeCarry carry;
    const bool cont = window_carry(rq.w, hist, carry);
    vhsdecode_gb300_decode_result_v1 dr{};
    dr.struct_size = sizeof(dr);
    decode_impl(sl->s, rq.w.samples, rq.w.sample_count, rq.w.max_fields, 0, &dr, nullptr, &carry);
    window_finish(sl->s, rq.w, carry, cont, dr, r, out_hist);
}

// A window picked by a worker, with its slot, history and result.
struct Item {
    Request rq;
    Slot* sl = nullptr;
    History hist, out_hist;
    vhsdecode_gb300_window_result_v1 r{};
    DecodeCarry carry;
    bool cont = false;
    vhsdecode_gb300_decode_result_v1 dr{};
};

void worker_main(vhsdecode_gb300_server* sv) {
    cudaSetDevice(sv->cfg.device_id);
    // cross-stream batching: the windows waiting when this worker becomes
    // free (up to max_batch) are demodulated by one persistent launch
    int max_batch = sv->cfg.max_batch > 1 ? (int)std::min<uint32_t>(sv->cfg.max_batch, 16u) : 1;
    BatchScratch bs;
    cudaStream_t bstream = nullptr;
    if (max_batch > 1) {
        try {
            bs.init(max_batch);
            ck(cudaStreamCreateWithFlags(&bstream, cudaStreamNonBlocking), "cudaStreamCreate");
        } catch (...) {
            max_batch = 1;   // no batching resources: windows decode one at a time
        }
    }
    for (;;) {
        std::vector<Item> items;
        std::vector<Slot*> release;
        {
            Item first;
            std::unique_lock<std::mutex> lk(sv->m);
            sv->cv_work.wait(lk, [&] { return sv->stop || pick(sv, first.rq, first.sl, release); });
            if (!first.sl) break;   // stopping
            items.push_back(first);
            if (max_batch > 1 && window_decim(first.rq.w) == 1) {
                for (;;) {
                    if ((int)items.size() >= max_batch) break;
                    Item more;
                    if (!pick(sv, more.rq, more.sl, release, true)) break;
                    items.push_back(more);
                }
            }
            for (Item& it : items) it.hist = sv->streams[it.rq.w.stream_id];
        }
        for (Slot* old : release) destroy_slot(old);
        for (Item& it : items) {
            it.r.struct_size = sizeof(it.r);
            it.r.ticket = it.rq.ticket;
            it.r.stream_id = it.rq.w.stream_id;
            it.r.sample_count = it.rq.w.sample_count;
            it.out_hist = it.hist;
            it.out_hist.busy = false;
        }
        auto t_start = Clock::now();
        std::vector<Clock::time_point> t_end(items.size());
        if (items.size() == 1) {
            Item& it = items[0];
            it.r.status = guard([&] {
                if (!it.sl->s) create_slot(sv, it.sl);
                run_window(it.sl, it.rq, it.hist, it.r, it.out_hist);
                return VHSDECODE_GB300_STATUS_OK;
            });
            t_end[0] = Clock::now();
        } else {
            int32_t st = guard([&] {
                for (Item& it : items)
                    if (!it.sl->s) create_slot(sv, it.sl);
                std::vector<BatchWindow> wins;
                for (Item& it : items) {
                    it.cont = window_carry(it.rq.w, it.hist, it.carry);
                    it.dr = vhsdecode_gb300_decode_result_v1{};
                    it.dr.struct_size = sizeof(it.dr);
                    wins.push_back(BatchWindow{it.sl->s, static_cast<const int16_t*>(it.rq.w.samples),
                                               it.rq.w.sample_count, it.rq.w.max_fields, &it.carry, &it.dr});
                }
                decode_batched(wins, bs, bstream);
                for (size_t i = 0; i < items.size(); i++) {
                    Item& it = items[i];
                    window_finish(it.sl->s, it.rq.w, it.carry, it.cont, it.dr, it.r, it.out_hist);
                    t_end[i] = Clock::now();
                }
                return VHSDECODE_GB300_STATUS_OK;
            });
            for (size_t i = 0; i < items.size(); i++) {
                items[i].r.status = st;
                if (st != VHSDECODE_GB300_STATUS_OK) t_end[i] = Clock::now();
            }
        }
        {
            std::lock_guard<std::mutex> lk(sv->m);
            for (size_t i = 0; i < items.size(); i++) {
                Item& it = items[i];
                it.r.queue_ms = ms_between(it.rq.submitted, t_start);
                it.r.decode_ms = ms_between(t_start, t_end[i]);
                it.r.latency_ms = ms_between(it.rq.submitted, t_end[i]);
                it.r.batched = (uint32_t)items.size();
                if (it.r.status != VHSDECODE_GB300_STATUS_OK) it.out_hist.valid = false;
                History& h = sv->streams[it.rq.w.stream_id];
                h = it.out_hist;
                h.busy = false;
                Slot* sl = it.sl;
                if (!sl->s) {   // creation failed: drop the reservation
                    sv->slots.erase(std::find(sv->slots.begin(), sv->slots.end(), sl));
                    sv->used -= sl->bytes;
                    delete sl;
                } else {
                    sl->busy = false;
                    sl->last_used = t_end[i];
                }
                sv->done[it.rq.ticket] = it.r;
            }
        }
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
    if (bstream) cudaStreamDestroy(bstream);
}

bool supported(const vhsdecode_gb300_window_v1& w) {
    return (w.profile == VHSDECODE_GB300_PROFILE_PAL || w.profile == VHSDECODE_GB300_PROFILE_NTSC) &&
           w.tape_speed <= VHSDECODE_GB300_TAPE_SPEED_EP &&
           (w.tape_format == VHSDECODE_GB300_TAPE_FORMAT_VHS || w.tape_format == VHSDECODE_GB300_TAPE_FORMAT_SVHS) &&
           w.sample_rate_mhz >= 10.0 && w.sample_rate_mhz <= 100.0 && w.decimation <= 2 &&
           (w.decimation != 2 || w.sample_rate_mhz <= 50.0);
}

}  // namespace

extern "C" {

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_create(
    const vhsdecode_gb300_server_config_v1* config, vhsdecode_gb300_server** server) {
    return guard([&] {
        if (!config || !server) throw Failure(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        *server = nullptr;
        if (config->struct_size != sizeof(vhsdecode_gb300_server_config_v1))
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "server config struct_size mismatch");
        if (config->max_window_samples < (uint64_t)kBlock)
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "max_window_samples below one block");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw Failure(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
        }
        if (config->device_id < 0 || config->device_id >= ndev)
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device_id out of range");
        ck(cudaSetDevice(config->device_id), "cudaSetDevice");
        auto* sv = new vhsdecode_gb300_server();
        sv->cfg = *config;
        size_t fr = 0, total = 0;
        ck(cudaMemGetInfo(&fr, &total), "cudaMemGetInfo");
        sv->budget = config->memory_budget_bytes ? (size_t)config->memory_budget_bytes : (size_t)(0.8 * (double)fr);
        uint32_t nw = config->workers ? config->workers : 4;
        for (uint32_t i = 0; i < nw; i++) sv->workers.emplace_back(worker_main, sv);
        *server = sv;
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_submit(
    vhsdecode_gb300_server* server, const vhsdecode_gb300_window_v1* window, uint64_t* ticket) {
    return guard([&] {
        if (!server || !window || !ticket) throw Failure(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (window->struct_size != sizeof(vhsdecode_gb300_window_v1))
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "window struct_size mismatch");
        if (!window->samples && window->sample_count)
            throw Failure(VHSDECODE_GB300_STATUS_NULL_POINTER, "null samples");
        if (!supported(*window))
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                          "unsupported window format (PAL or NTSC VHS SP, 10-100 MSPS)");
        if (window->sample_count > server->cfg.max_window_samples)
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "window longer than max_window_samples");
        std::lock_guard<std::mutex> lk(server->m);
        if (server->stop) throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "server is shutting down");
        Request rq;
        rq.ticket = server->next_ticket++;
        rq.w = *window;
        rq.submitted = Clock::now();
        server->queue.push_back(rq);
        *ticket = rq.ticket;
        server->cv_work.notify_one();
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_wait(
    vhsdecode_gb300_server* server, uint64_t ticket, vhsdecode_gb300_window_result_v1* result) {
    return guard([&] {
        if (!server || !result) throw Failure(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (result->struct_size != sizeof(vhsdecode_gb300_window_result_v1))
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "result struct_size mismatch");
        std::unique_lock<std::mutex> lk(server->m);
        if (ticket == 0 || ticket >= server->next_ticket)
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unknown ticket");
        server->cv_done.wait(lk, [&] { return server->done.count(ticket) > 0; });
        *result = server->done[ticket];
        server->done.erase(ticket);
        return result->status;
    });
}

VHSDECODE_GB300_API void VHSDECODE_GB300_CALL vhsdecode_gb300_server_destroy(vhsdecode_gb300_server* server) {
    if (!server) return;
    {
        std::lock_guard<std::mutex> lk(server->m);
        server->stop = true;
        for (const Request& rq : server->queue) {
            vhsdecode_gb300_window_result_v1 r{};
            r.struct_size = sizeof(r);
            r.status = VHSDECODE_GB300_STATUS_CANCELLED;
            r.ticket = rq.ticket;
            r.stream_id = rq.w.stream_id;
            server->done[rq.ticket] = r;
        }
        server->queue.clear();
    }
    server->cv_work.notify_all();
    server->cv_done.notify_all();
    for (auto& t : server->workers) t.join();
    for (Slot* sl : server->slots) destroy_slot(sl);
    delete server;
}

}  // extern "C"
