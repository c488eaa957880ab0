// als_logger.hpp — header-only C++ face of the library's event log with the reference's logger
// interface (logger.h:7-48), so a caller written against that global compiles unchanged:
//
//   logger g_logger;
//   g_logger.init(log_folder);                                   // logger.cpp:56-73
//   g_logger.run_iter = i + 1;
//   g_logger.event_started(logger::EVENT_TYPE::MF_MODEL_TRAINING);
//   g_logger.event_finished(logger::EVENT_TYPE::MF_MODEL_TRAINING, true);
//   g_logger.log("final RMSE test: ...", true);
//   g_logger.save();                                             // logger.cpp:145-153
//
// The CSV and its columns are written by the library (als_log_* in als_gb300.h); run_iter and
// als_iter stay public fields and are handed to the log before every call.  Errors throw
// als_gb300_error.
#pragma once

#include <cstddef>
#include <string>

#include "als_error.hpp"
#include "als_gb300.h"

struct logger {
    enum class EVENT_TYPE { ALS_UPDATE_U = 0, ALS_UPDATE_V, ALS_ITER, MF_MODEL_TRAINING };

    logger() = default;
    ~logger() {
        if (lg_) als_log_destroy(lg_);
    }
    logger(const logger &) = delete;
    logger &operator=(const logger &) = delete;

    // Starts a new CSV (header + "init logger"); a second init starts over.
    void init(const std::string &log_folder_) {
        if (lg_) als_log_destroy(lg_);
        lg_ = nullptr;
        check(als_log_create(log_folder_.c_str(), &lg_));
        log_folder = log_folder_;
        log_name = als_log_name(lg_);
    }
    void log(const std::string &text, bool write_cout) {
        sync();
        check(als_log_text(lg_, text.c_str(), write_cout ? 1 : 0));
    }
    void event_started(EVENT_TYPE t) {
        sync();
        check(als_log_event_started(lg_, (int32_t)t));
    }
    void event_finished(EVENT_TYPE t, bool write_cout) {
        sync();
        check(als_log_event_finished(lg_, (int32_t)t, write_cout ? 1 : 0));
    }
    void save() { check(als_log_save(lg_, nullptr)); }
    void save(const std::string &log_path) { check(als_log_save(lg_, log_path.c_str())); }

    // The CSV so far (not in the reference, which keeps it in a stringstream member).
    std::string contents() const {
        size_t n = 0;
        check(als_log_contents(lg_, nullptr, &n));
        std::string s(n, '\0');
        check(als_log_contents(lg_, &s[0], &n));
        s.resize(n ? n - 1 : 0);
        return s;
    }

    static std::string to_string(EVENT_TYPE t) {
        switch (t) {
            case EVENT_TYPE::ALS_UPDATE_U: return "ALS_UPDATE_U";
            case EVENT_TYPE::ALS_UPDATE_V: return "ALS_UPDATE_V";
            case EVENT_TYPE::ALS_ITER: return "ALS_ITER";
            case EVENT_TYPE::MF_MODEL_TRAINING: return "MF_MODEL_TRAINING";
        }
        return "UNKNOWN";
    }

    // The library object, for als_model::set_logger; the iteration fields are pushed first and
    // read back by pull() after the library wrote lines of its own.
    als_log *handle() {
        sync();
        return lg_;
    }
    void pull() {
        int64_t r = 0, a = 0;
        check(als_log_get_iters(lg_, &r, &a));
        run_iter = (size_t)r;
        als_iter = (size_t)a;
    }

    std::string log_folder;
    std::string log_name;
    size_t run_iter = 0;
    size_t als_iter = 0;

private:
    void sync() {
        if (!lg_) throw als_gb300_error(ALS_ERR_INVALID_ARG, "logger used before init()");
        check(als_log_set_iters(lg_, (int64_t)run_iter, (int64_t)als_iter));
    }
    static void check(als_status s) { als_gb300_detail::check(s); }
    als_log *lg_ = nullptr;
};
