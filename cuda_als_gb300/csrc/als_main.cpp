// als_main.cpp — the reference's command-line driver (main.cpp:18-123) on this library:
//
//   als_gb300_main <config.ini> [model_out]
//
// Reads the reference's INI keys ([data] data_folder, m, n, nnz_train, nnz_test; [als] f,
// lambda, als_iters, als_calculate_vtvs_type, als_solve_type, m_batches, n_batches; [general]
// als_runs, log_folder) plus the optional [als_gb300] section (precision, solver options, and
// iter_rmse = 1 for the per-iteration test RMSE lines, model_path for the libmf output), loads
// the reference's .bin files, trains als_runs models and writes the event log the reference's
// USE_LOGGER build writes, with the same lines in the same order:
//   parameters, "host train and test ratings loaded", per run MF_MODEL_TRAINING around
//   construction + train (with train()'s own lines), "final RMSE test: <%f>", and when
//   als_runs == 1 the libmf model ("saved model in cumf_sgd libmf format"), then
//   "all als runs done"; the CSV is saved to <log_folder>/<UTC date>_debug=false.csv.
// The model is written only when a path is given (argv[2] or [als_gb300] model_path): the
// reference writes it to a path fixed in its source (main.cpp:108-112).
// Exit status: 0 done; 1 the INI cannot be read (main.cpp:23-26); 2 usage; 3 a library error,
// printed as "ERROR <STATUS>: <message>" after saving the log so far.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

#include "als_logger.hpp"
#include "als_model.hpp"

static std::string ini_string(const char *path, const char *section, const char *key) {
    char buf[4096];
    als_gb300_detail::check(als_ini_get(path, section, key, buf, sizeof(buf)));
    return buf;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <config.ini> [model_out]\n", argv[0]);
        return 2;
    }
    const std::string ini_path = argv[1];
    als_config cfg;
    int64_t m = 0, n = 0, nnz_train = 0, nnz_test = 0;
    int32_t als_runs = 0;
    char folder[4096];
    if (als_config_from_ini(ini_path.c_str(), &cfg, &m, &n, &nnz_train, &nnz_test, &als_runs,
                            folder, sizeof(folder)) != ALS_OK) {
        std::cout << "Can't load " << ini_path << "\n";
        return 1;
    }
    const std::string data_folder = folder;
    logger g_logger;
    try {
        const std::string log_folder = ini_string(argv[1], "general", "log_folder");
        const bool iter_rmse = ini_string(argv[1], "als_gb300", "iter_rmse") == "1";
        std::string model_path = argc > 2 ? argv[2] : ini_string(argv[1], "als_gb300", "model_path");
        const auto vtvs = (als_model::CALCULATE_VTVS_TYPE)cfg.calculate_vtvs_type;
        const auto solve = (als_model::SOLVE_TYPE)cfg.solve_type;

        std::cout << std::fixed;
        g_logger.init(log_folder);
        std::stringstream ss;  // main.cpp:54-60 (default float format for lambda)
        ss << "m=" << m << " n=" << n << " f=" << cfg.f << " nnz_train=" << nnz_train
           << " nnz_test=" << nnz_test << " lambda=" << cfg.lambda << " als_iters=" << cfg.iters
           << " data_folder=" << data_folder << " als_runs=" << als_runs
           << " log_folder=" << log_folder
           << " als_calculate_vtvs_type=" << als_model::to_string(vtvs)
           << " als_solve_type=" << als_model::to_string(solve)
           << " smem_col_cnt=" << cfg.smem_col_cnt;
        g_logger.log(ss.str(), true);

        try {
            // main.cpp:68-75
            const std::string &d = data_folder;
            host_sparse_matrix train((size_t)m, (size_t)n, (size_t)nnz_train);
            train.load_csc(d + "/R_train_csc.data.bin", d + "/R_train_csc.indices.bin",
                           d + "/R_train_csc.indptr.bin");
            train.load_csr(d + "/R_train_csr.data.bin", d + "/R_train_csr.indptr.bin",
                           d + "/R_train_csr.indices.bin");
            train.load_coo(d + "/R_train_csr.data.bin", d + "/R_train_coo.row.bin",
                           d + "/R_train_csr.indices.bin");
            host_sparse_matrix test((size_t)m, (size_t)n, (size_t)nnz_test);
            test.load_coo(d + "/R_test_coo.data.bin", d + "/R_test_coo.row.bin",
                          d + "/R_test_coo.col.bin");
            g_logger.log("host train and test ratings loaded", true);

            // main.cpp:82-114
            for (int32_t i = 0; i < als_runs; ++i) {
                g_logger.event_started(logger::EVENT_TYPE::MF_MODEL_TRAINING);
                g_logger.run_iter = (size_t)i + 1;
                als_model model(train, test, cfg);
                g_logger.log("als model constructor done", true);
                model.set_logger(g_logger, iter_rmse, true);
                model.train();
                g_logger.event_finished(logger::EVENT_TYPE::MF_MODEL_TRAINING, true);
                g_logger.log("final RMSE test: " + std::to_string(model.rsme_test()), true);
                if (als_runs == 1 && !model_path.empty()) {
                    model.save_libmf(model_path.c_str());
                    g_logger.log("saved model in cumf_sgd libmf format", true);
                }
            }
            g_logger.run_iter = 0;
            g_logger.log("all als runs done", true);
            g_logger.save();
        } catch (const als_gb300_error &) {
            try {
                g_logger.save();  // the lines so far
            } catch (const als_gb300_error &) {
            }
            throw;
        }
    } catch (const als_gb300_error &e) {
        std::cout << "ERROR " << e.what() << std::endl;
        return 3;
    }
    return 0;
}
