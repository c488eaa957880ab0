// Replays a script of logger calls on the reference's own logger (logger.h / logger.cpp of
// vserdyuk/cuda_als, compiled from its sources by oracle/build.py into oracle/_ref/), so that
// the tests can pin the event log's CSV format and stdout echo to the real thing.
// TEST INFRASTRUCTURE ONLY: the library never links or runs this.
//
// usage: ref_logger <out.csv> < script
// script lines (one call each, as the reference's main.cpp / als_model.cu make them):
//   log <0|1> <text...>        g_logger.log(text, write_cout)
//   start <event>              g_logger.event_started(EVENT_TYPE(event))
//   finish <event> <0|1>       g_logger.event_finished(EVENT_TYPE(event), write_cout)
//   iters <run_iter> <als_iter>  set the two public fields
//   sleep_us <n>               wait n microseconds (to make the timestamp columns differ)
#include <chrono>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>

#include "logger.h"

logger g_logger;

int main(int argc, char **argv) {
    if (argc < 2) {
        std::cerr << "usage: ref_logger <out.csv> < script\n";
        return 2;
    }
    std::cout << std::fixed;  // main.cpp:52
    g_logger.init(".");
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string op;
        in >> op;
        if (op == "log") {
            int c = 0;
            in >> c;
            std::string text;
            std::getline(in, text);
            if (!text.empty() && text[0] == ' ') text.erase(0, 1);
            g_logger.log(text, c != 0);
        } else if (op == "start") {
            int e = 0;
            in >> e;
            g_logger.event_started((logger::EVENT_TYPE)e);
        } else if (op == "finish") {
            int e = 0, c = 0;
            in >> e >> c;
            g_logger.event_finished((logger::EVENT_TYPE)e, c != 0);
        } else if (op == "iters") {
            in >> g_logger.run_iter >> g_logger.als_iter;
        } else if (op == "sleep_us") {
            long us = 0;
            in >> us;
            std::this_thread::sleep_for(std::chrono::microseconds(us));
        }
    }
    g_logger.save(argv[1]);
    return 0;
}
