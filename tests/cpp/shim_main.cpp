// The reference's main.cpp flow (main.cpp:60-105) against include/als_model.hpp: load the .bin
// files by their reference names, construct als_model, train, print the test RMSE, save the model.
// argv: folder m n nnz_train nnz_test f lambda iters vtvs solve [model_out]
// Exit 0 on success, 3 with "ERROR <status>: <message>" on an als_gb300_error.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "als_model.hpp"

int main(int argc, char **argv) {
    if (argc < 11) {
        std::fprintf(stderr, "usage: %s folder m n nnz_train nnz_test f lambda iters vtvs solve [out]\n",
                     argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    const size_t m = std::strtoull(argv[2], nullptr, 10), n = std::strtoull(argv[3], nullptr, 10);
    const size_t nnz_train = std::strtoull(argv[4], nullptr, 10);
    const size_t nnz_test = std::strtoull(argv[5], nullptr, 10);
    const int f = std::atoi(argv[6]);
    const float lambda = (float)std::atof(argv[7]);
    const int iters = std::atoi(argv[8]);
    const auto vtvs = (als_model::CALCULATE_VTVS_TYPE)std::atoi(argv[9]);
    const auto solve = (als_model::SOLVE_TYPE)std::atoi(argv[10]);
    try {
        host_sparse_matrix train(m, n, nnz_train);
        train.load_csc(dir + "/R_train_csc.data.bin", dir + "/R_train_csc.indices.bin",
                       dir + "/R_train_csc.indptr.bin");
        train.load_csr(dir + "/R_train_csr.data.bin", dir + "/R_train_csr.indptr.bin",
                       dir + "/R_train_csr.indices.bin");
        train.load_coo(dir + "/R_train_csr.data.bin", dir + "/R_train_coo.row.bin",
                       dir + "/R_train_csr.indices.bin");
        host_sparse_matrix test(m, n, nnz_test);
        test.load_coo(dir + "/R_test_coo.data.bin", dir + "/R_test_coo.row.bin",
                      dir + "/R_test_coo.col.bin");
        als_model model(train, test, f, lambda, iters, vtvs, solve, 32, 1, 1);
        model.train();
        std::printf("rmse_test %.9f\nrmse_train %.9f\nsolve %s\nvtvs %s\nU0 %.9g\nV0 %.9g\n",
                    model.rsme_test(), model.rsme_train(),
                    als_model::to_string(solve).c_str(), als_model::to_string(vtvs).c_str(),
                    (double)model.h_UT[0], (double)model.h_VT[0]);
        if (argc > 11) model.save_libmf(argv[11]);
    } catch (const als_gb300_error &e) {
        std::printf("ERROR %s\n", e.what());
        return 3;
    }
    return 0;
}
