// eventlog.cpp — the timing CSV of the reference's logger (logger.h:7-48, logger.cpp:42-163),
// as a C-ABI object instead of a process-wide global, and the lines als_train writes into it.
//
// Columns and meaning are kept so that the reference's analysis queries (averages of `elapsed`
// per text, of `event_elapsed` per event) read these logs unchanged:
//   log_name,id,run_iter,als_iter,prev_ts,curr_ts,elapsed,event_elapsed,text
// * a text line advances prev_ts and then prints it, so its prev_ts column equals curr_ts and
//   `elapsed` is the time since the previous text line (logger.cpp:75-87);
// * an event-finished line prints the last text line's time as prev_ts, does not advance it, and
//   carries event_elapsed = now - the event's start (logger.cpp:108-143).
// Timestamps are wall-clock seconds since the epoch with microsecond resolution (gettimeofday in
// the reference, logger.cpp:42-46), printed with 6 decimals (std::fixed).
#include <chrono>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>

#include "handle.h"
#include "internal.h"

using als::set_global_error;

struct als_log {
    std::string folder, name;
    std::ostringstream ss;
    double prev_ts = 0.0;
    double started[4] = {0.0, 0.0, 0.0, 0.0};
    int64_t next_id = 0, run_iter = 0, als_iter = 0;
    mutable std::mutex mu;
};

namespace {

const char *event_name(int32_t e) {
    switch (e) {
        case ALS_EVENT_UPDATE_U: return "ALS_UPDATE_U";
        case ALS_EVENT_UPDATE_V: return "ALS_UPDATE_V";
        case ALS_EVENT_ITER: return "ALS_ITER";
        case ALS_EVENT_MF_MODEL_TRAINING: return "MF_MODEL_TRAINING";
        default: return "UNKNOWN";
    }
}

double now_seconds() {
    const auto us = std::chrono::duration_cast<std::chrono::microseconds>(
                        std::chrono::system_clock::now().time_since_epoch())
                        .count();
    return (double)(us / 1000000) + (double)(us % 1000000) * 1e-6;
}

std::string utc_stamp() {
    const std::time_t t = std::time(nullptr);
    std::tm tm{};
    gmtime_r(&t, &tm);
    char buf[32];
    std::strftime(buf, sizeof(buf), "%Y%m%d_%H%M%S", &tm);
    return buf;
}

void echo(const als_log *lg, double elapsed, const double *event_elapsed, const std::string &text) {
    std::ostringstream o;
    o << std::fixed << "run iter: " << lg->run_iter << " als iter: " << lg->als_iter
      << " elapsed: " << elapsed;
    if (event_elapsed) o << " event elapsed: " << *event_elapsed;
    o << " " << text << "\n";
    std::cout << o.str() << std::flush;
}

}  // namespace

// Internal entry points for api.cpp (the training lines).
namespace als {

void log_text(als_log *lg, const std::string &text, bool write_cout) {
    std::lock_guard<std::mutex> lock(lg->mu);
    const double curr = now_seconds();
    const double elapsed = curr - lg->prev_ts;
    lg->prev_ts = curr;
    lg->ss << lg->name << "," << lg->next_id++ << "," << lg->run_iter << "," << lg->als_iter
           << "," << lg->prev_ts << "," << curr << "," << elapsed << ",," << text << "\n";
    if (write_cout) echo(lg, elapsed, nullptr, text);
}

void log_event(als_log *lg, int32_t event, bool finished, bool write_cout) {
    std::lock_guard<std::mutex> lock(lg->mu);
    const double curr = now_seconds();
    if (!finished) {
        lg->started[event] = curr;
        return;
    }
    const double elapsed = curr - lg->prev_ts;
    const double event_elapsed = curr - lg->started[event];
    lg->started[event] = 0.0;
    const std::string text = std::string("event ") + event_name(event) + " finished";
    lg->ss << lg->name << "," << lg->next_id++ << "," << lg->run_iter << "," << lg->als_iter
           << "," << lg->prev_ts << "," << curr << "," << elapsed << "," << event_elapsed << ","
           << text << "\n";
    if (write_cout) echo(lg, elapsed, &event_elapsed, text);
}

void log_set_als_iter(als_log *lg, int64_t als_iter) {
    std::lock_guard<std::mutex> lock(lg->mu);
    lg->als_iter = als_iter;
}

}  // namespace als

extern "C" als_status als_log_create(const char *log_folder, als_log **out) {
    if (!out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    als_log *lg = new (std::nothrow) als_log;
    if (!lg) return set_global_error(ALS_ERR_OUT_OF_MEMORY, "als_log_create: out of memory");
    lg->folder = log_folder ? log_folder : "";
    lg->name = utc_stamp() + "_debug=false.csv";
    lg->prev_ts = now_seconds();
    lg->ss << std::fixed;
    lg->ss << "log_name,id,run_iter,als_iter,prev_ts,curr_ts,elapsed,event_elapsed,text\n";
    als::log_text(lg, "init logger", false);
    *out = lg;
    return ALS_OK;
}

extern "C" als_status als_log_destroy(als_log *lg) {
    delete lg;
    return ALS_OK;
}

extern "C" als_status als_log_text(als_log *lg, const char *text, int32_t write_cout) {
    if (!lg || !text) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    als::log_text(lg, text, write_cout != 0);
    return ALS_OK;
}

static bool valid_event(int32_t e) { return e >= ALS_EVENT_UPDATE_U && e <= ALS_EVENT_MF_MODEL_TRAINING; }

extern "C" als_status als_log_event_started(als_log *lg, int32_t event) {
    if (!lg || !valid_event(event)) return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    als::log_event(lg, event, false, false);
    return ALS_OK;
}

extern "C" als_status als_log_event_finished(als_log *lg, int32_t event, int32_t write_cout) {
    if (!lg || !valid_event(event)) return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    als::log_event(lg, event, true, write_cout != 0);
    return ALS_OK;
}

extern "C" als_status als_log_set_iters(als_log *lg, int64_t run_iter, int64_t als_iter) {
    if (!lg || run_iter < 0 || als_iter < 0)
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    std::lock_guard<std::mutex> lock(lg->mu);
    lg->run_iter = run_iter;
    lg->als_iter = als_iter;
    return ALS_OK;
}

extern "C" als_status als_log_get_iters(const als_log *lg, int64_t *run_iter, int64_t *als_iter) {
    if (!lg) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lock(lg->mu);
    if (run_iter) *run_iter = lg->run_iter;
    if (als_iter) *als_iter = lg->als_iter;
    return ALS_OK;
}

extern "C" const char *als_log_name(const als_log *lg) { return lg ? lg->name.c_str() : ""; }

extern "C" als_status als_log_contents(const als_log *lg, char *buf, size_t *len) {
    if (!lg || !len) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::string s;
    {
        std::lock_guard<std::mutex> lock(lg->mu);
        s = lg->ss.str();
    }
    const size_t need = s.size() + 1;
    if (buf) {
        if (*len < need) {
            *len = need;
            return set_global_error(ALS_ERR_INVALID_ARG, "als_log_contents: buffer too small");
        }
        std::memcpy(buf, s.c_str(), need);
    }
    *len = need;
    return ALS_OK;
}

extern "C" als_status als_log_save(const als_log *lg, const char *path) {
    if (!lg) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    const std::string p = path ? std::string(path)
                               : (lg->folder.empty() ? lg->name : lg->folder + "/" + lg->name);
    std::string s;
    {
        std::lock_guard<std::mutex> lock(lg->mu);
        s = lg->ss.str();
    }
    std::ofstream out(p, std::ios::binary);
    if (!out) return set_global_error(ALS_ERR_IO, p + ": cannot open for writing");
    out.write(s.data(), (std::streamsize)s.size());
    if (!out) return set_global_error(ALS_ERR_IO, p + ": write failed");
    return ALS_OK;
}

extern "C" als_status als_set_log(als_handle *h, als_log *lg, int32_t iter_rmse,
                                  int32_t write_cout) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    h->log = lg;
    h->log_iter_rmse = iter_rmse != 0;
    h->log_cout = write_cout != 0;
    return ALS_OK;
}
