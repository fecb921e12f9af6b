// mirror_driver.cpp -- the reference's Signal1D driver sequence (examples/test_signal1D/
// test_signal1D.cpp:188-288: data, decomposition, model, TSSolver, solve, save) written against
// include/pasc/pasc_gb300.hpp; used by tests/test_cpp_mirror.py.
//
//   mirror_driver --host-checks <dir>              checks that need no GPU
//   mirror_driver <data.bin> <K> <epssqr> <prefix>  solve on GPU 0, print L, theta, iterations
//   mirror_driver --image <data.bin> <width> <height> <K> <epssqr> <prefix>
//                                                   the test_image sequence (examples/test_image/
//                                                   test_image.cpp:156-221): grid graph, T = 1
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "pasc/pasc_gb300.hpp"

using namespace pasc_gb300;

static int host_checks(const std::string &dir)
{
    // PETSc binary round trip
    std::vector<double> v = {1.5, -2.25, 3.0e10, 0.0, -1e-300};
    save_vec(dir + "/roundtrip.bin", v);
    if (load_vec(dir + "/roundtrip.bin") != v) {
        std::printf("roundtrip FAILED\n");
        return 1;
    }
    std::printf("roundtrip ok\n");
    // the seeded uniforms of the default gamma0
    const std::vector<double> u = uniform(13, 0, 5);
    std::printf("uniform");
    for (double x : u) std::printf(" %.17g", x);
    std::printf("\n");
    // R > 1 nodes without a graph: disjoint nodes; a grid graph's edges
    {
        Decomposition d(100, 2, 3, 1, 1);
        BGMGraphGrid2D grid(4, 3);
        grid.process_grid();
        std::printf("R=2 nodes %d edges %d grid %d %d\n", d.get_graph()->get_n(), d.get_graph()->get_m(), grid.get_m(),
                    grid.get_m_max());
    }
    // data preprocessing on the host copy
    {
        Signal1DData sd(std::vector<double>{-3.0, 0.0, 1.0, 5.0});
        sd.cutdata(-1.0, 2.0);
        sd.scaledata(0.0, 1.0);
        std::printf("scaled");
        for (double x : sd.get_datavector()) std::printf(" %.17g", x);
        sd.unscaledata(0.0, 1.0);
        std::printf("\nunscaled");
        for (double x : sd.get_datavector()) std::printf(" %.17g", x);
        std::printf("\n");
    }
    // errors become exceptions
    try {
        Decomposition d(100, 2, 3, 2, 1);
        std::printf("xdim=2 graph accepted FAILED\n");
        return 1;
    } catch (const Error &e) {
        std::printf("xdim=2 code %d\n", e.code());
    }
    try {
        Problem p(0, 3, 1.0);
        std::printf("T=0 accepted FAILED\n");
        return 1;
    } catch (const Error &e) {
        std::printf("T=0 code %d\n", e.code());
    }
    return 0;
}

int main(int argc, char **argv)
{
    try {
        if (argc == 3 && std::string(argv[1]) == "--host-checks") return host_checks(argv[2]);
        if (argc == 8 && std::string(argv[1]) == "--image") {
            const int width = std::atoi(argv[3]), height = std::atoi(argv[4]), K = std::atoi(argv[5]);
            BGMGraphGrid2D graph(width, height);
            graph.process_grid();
            Decomposition decomposition(1, graph, K, 1, 1);
            ImageData mydata(decomposition, argv[2], width, height);
            GraphH1FEMModel mymodel(mydata, std::atof(argv[6]));
            TSSolver mysolver(mydata, 1, {{"spgqpsolver_m", 10}, {"spgqpsolver_eps", 1e-10}});
            mysolver.solve();
            std::printf("L %.17g\n", mysolver.get_L());
            std::printf("theta");
            for (double t : mydata.get_thetavector()) std::printf(" %.17g", t);
            std::printf("\n");
            mydata.saveImage(argv[7]);
            return 0;
        }
        if (argc != 5) {
            std::fprintf(stderr, "usage: %s <data.bin> <K> <epssqr> <prefix> | --host-checks <dir>\n", argv[0]);
            return 2;
        }
        const int K = std::atoi(argv[2]);
        const double epssqr = std::atof(argv[3]);
        Signal1DData mydata(argv[1]);
        mydata.set_decomposition(Decomposition(mydata.get_Tpreliminary(), 1, K, 1, 1));
        GraphH1FEMModel mymodel(mydata, epssqr);
        // the sweep kernel is otherwise chosen by timing, per process; pinned so that this run
        // and the Python one make the same FP32 roundings
        mymodel.problem().set_sweep_variant(1);
        TSSolver mysolver(mydata, 1, {{"spgqpsolver_m", 10}, {"spgqpsolver_eps", 1e-6}});
        mysolver.solve();
        std::printf("L %.17g\n", mysolver.get_L());
        std::printf("aic %.17g\n", mydata.get_aic());
        std::printf("theta");
        for (double t : mydata.get_thetavector()) std::printf(" %.17g", t);
        std::printf("\nspg_it %d\n", mysolver.get_gammasolver().get_it());
        mydata.saveSignal1D(argv[4]);
        return 0;
    } catch (const Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
}
