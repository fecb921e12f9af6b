// gb300_backend_driver.cpp -- runs the reference's OWN generic solvers, SPGQPSolver<GB300Vec>
// and TSSolver<GB300Vec>, with the GB300 backend of include/pasc/gb300_backend.hpp: every vector
// operation of the reference's loops goes through the C ABI to the GPU.
//
// Test infrastructure: it is compiled from the PASC_inference headers (generic templates,
// unmodified) and the shims of oracle/ref_shim, which stand in for the reference's PETSc/MPI
// common layer (console, options, one-rank decomposition, TSData).  oracle/build_ref.sh writes
// it out as one translation unit with the reference's headers inlined (oracle/_ref/backend/),
// which tests/test_gpu_backend.py compiles and runs on the GPU machine.
//
// usage: gb300_backend_driver <in.bin> <out.bin>
//   in.bin : int32 mode (0 SPGQPSolver, 1 TSSolver), int32 T, int32 K, then FP64: epssqr,
//            spg_maxit, spg_eps, spg_m, spg_stop_difff, ts_maxit, ts_eps, data[T], theta[K],
//            gamma[K*T] (mode 0: the start point, interleaved t*K + k; mode 1: what set_random
//            gives, blocked k*T + t, permuted on the device before the solve)
//   out.bin: FP64 fx_or_L, it, hessmult_or_it_sum, theta[K], gamma[K*T] (interleaved)
#include "general/common/common.h"
#include "general/data/qpdata.h"
#include "general/data/simpledata.h"
#include "general/algebra/feasibleset/simplex_local.h"
#include "general/algebra/matrix/blockgraphsparse.h"
#include "general/solver/spgqpsolver.h"
#include "general/solver/simplesolver.h"
#include "general/model/tsmodel.h"
#include "general/data/tsdata.h"
#include "general/solver/tssolver.h"

#include "pasc/gb300_backend.hpp"

#include <cstdio>

namespace pascinference {
namespace common {
ConsoleOutput coutMaster;
ConsoleOutput coutAll;
ConsoleArg consoleArg;
GlobalManagerClass GlobalManager;
}  // namespace common
namespace algebra {
std::vector<double> refshim_random_source;
}
}  // namespace pascinference

using namespace pascinference;
using V = algebra::GB300Vec;

class DriverTSSolver : public TSSolver<V> {
  public:
    DriverTSSolver(TSData<V> &d) : TSSolver<V>(d, 1) {}
    int it_last_() const { return this->it_last; }
    int it_sum_() const { return this->it_sum; }
};

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    double opt[7];
    if (std::fread(hdr, sizeof(int), 3, f) != 3 || std::fread(opt, sizeof(double), 7, f) != 7) return 2;
    const int mode = hdr[0], T = hdr[1], K = hdr[2];
    const size_t N = (size_t)T * K;
    std::vector<double> data(T), theta(K), gamma(N);
    if (std::fread(data.data(), sizeof(double), T, f) != (size_t)T ||
        std::fread(theta.data(), sizeof(double), K, f) != (size_t)K ||
        std::fread(gamma.data(), sizeof(double), N, f) != N)
        return 2;
    std::fclose(f);
    const double epssqr = opt[0];
    consoleArg.overrides["spgqpsolver_maxit"] = opt[1];
    consoleArg.overrides["spgqpsolver_eps"] = opt[2];
    consoleArg.overrides["spgqpsolver_m"] = opt[3];
    consoleArg.overrides["spgqpsolver_stop_difff"] = opt[4];
    consoleArg.overrides["tssolver_maxit"] = opt[5];
    consoleArg.overrides["tssolver_eps"] = opt[6];
    consoleArg.overrides["tssolver_init_permute"] = 0;  // permuted on the device below

    double out3[3] = {0, 0, 0};
    std::vector<double> g_out(N), th_out(K);
    try {
        if (mode == 0) {
            Decomposition<V> dec(T, 1, K, 1, 1);
            BlockGraphSparseMatrix<V> A(dec, epssqr / (double)T, NULL);
            GeneralVector<V> x((long)N), b((long)N), dv((long)T), tv((long)K);
            x.upload(gamma);
            dv.upload(data);
            tv.upload(theta);
            pasc_gb300_residual_f64(dv.dev(), tv.dev(), b.dev(), T, K, -1.0 / (double)T, nullptr);
            QPData<V> qp;
            qp.set_A(&A);
            qp.set_b(&b);
            qp.set_x(&x);
            qp.set_x0(&x);
            SimplexFeasibleSet_Local<V> fs(T, K);
            qp.set_feasibleset(&fs);
            {
                SPGQPSolver<V> solver(qp);
                solver.solve();
                out3[0] = solver.get_fx();
                out3[1] = solver.get_it();
                out3[2] = solver.get_hessmult();
            }
            g_out = x.download();
            th_out = theta;
        } else {
            Decomposition<V> dec(T, 1, K, 1, 1);
            GeneralVector<V> dv((long)T), gv((long)N), tv((long)K);
            dv.upload(data);
            tv.upload(theta);
            gv.upload(gamma);
            algebra::gb300_random_source() = gamma;
            gv.permute_blocked(T, K);
            TSData<V> tsdata(dec, &dv, &gv, &tv);
            model::GB300H1FEMModel mymodel(tsdata, epssqr);
            {
                DriverTSSolver solver(tsdata);
                solver.solve();
                out3[0] = solver.get_L();
                out3[1] = solver.it_last_();
                out3[2] = solver.it_sum_();
            }
            g_out = gv.download();
            th_out = tv.download();
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "gb300_backend_driver: %s\n", e.what());
        return 1;
    }
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(out3, sizeof(double), 3, o);
    std::fwrite(th_out.data(), sizeof(double), K, o);
    std::fwrite(g_out.data(), sizeof(double), N, o);
    std::fclose(o);
    return 0;
}
