/*
 * Shim for the reference's general/common/common.h, used ONLY by oracle/build_ref.sh to
 * compile the reference's own solver templates (spgqpsolver.h, tssolver.h, spg_fs.cpp,
 * simplex_local.h, ...) without PETSc, MPI or Boost.  Test infrastructure, never shipped.
 *
 * It supplies the infrastructure those headers use -- console output, option lookup,
 * timers, logging macros, a global manager, a rank barrier and the few PETSc names that
 * appear in the generic template bodies -- backed by plain host arrays.
 */
#ifndef PASC_REFSHIM_COMMON_H
#define PASC_REFSHIM_COMMON_H

#include <sys/types.h>
#include <iostream>
#include <iomanip>
#include <typeinfo>
#include <cmath>
#include <math.h>
#include <string>
#include <fstream>
#include <sstream>
#include <stack>
#include <limits>
#include <map>
#include <vector>
#include <chrono>
#include <cstring>

namespace pascinference {
namespace common {

/* Console output that discards everything (the solvers print progress only in debug modes). */
class ConsoleOutput {
  public:
    template <class T> ConsoleOutput &operator<<(const T &) { return *this; }
    ConsoleOutput &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
    void push() {}
    void pop() {}
    void synchronize() {}
};
extern ConsoleOutput coutMaster;
extern ConsoleOutput coutAll;

/* Option lookup: every option takes its default unless the driver set an override. */
class ConsoleArg {
  public:
    std::map<std::string, double> overrides;
    template <class T, class U> bool set_option_value(const std::string &name, T *var, U def) {
        auto it = overrides.find(name);
        if (it != overrides.end()) { *var = (T)it->second; return true; }
        *var = (T)def;
        return false;
    }
    template <class T> bool set_option_value(const std::string &name, T *var) {
        auto it = overrides.find(name);
        if (it != overrides.end()) { *var = (T)it->second; return true; }
        return false;
    }
};
extern ConsoleArg consoleArg;

class Timer {
    double sum_ = 0.0, last_ = 0.0;
    std::chrono::steady_clock::time_point t0_;
    bool run_ = false;
  public:
    void restart() { sum_ = 0.0; last_ = 0.0; run_ = false; }
    void start() { t0_ = std::chrono::steady_clock::now(); run_ = true; }
    void stop() {
        if (!run_) return;
        last_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
        sum_ += last_;
        run_ = false;
    }
    double get_value_last() const { return last_; }
    double get_value_sum() const { return sum_; }
};

class MemoryCheck {
  public:
    static double get_virtual() { return 0.0; }
};

class GlobalManagerClass {
  public:
    int get_rank() const { return 0; }
    int get_size() const { return 1; }
};
extern GlobalManagerClass GlobalManager;

} /* namespace common */

namespace algebra {}
namespace data {}
namespace solver {}
namespace model {}
using namespace common;
using namespace algebra;
using namespace data;
using namespace solver;
using namespace model;

template <class VectorBase> void allbarrier() {}

} /* namespace pascinference */

#define LOG_FUNC_BEGIN
#define LOG_FUNC_END
#define LOG_FUNC_STATIC_BEGIN
#define LOG_FUNC_STATIC_END
#define LOG_IT(x)
#define LOG_FX(x)
#define LOG_FX2(x, n)
#define LOG_DIRECT(x)
#define PetscSqrtReal(x) std::sqrt(x)

/* PETSc names that appear in generic template bodies (tssolver.h gammavector_permute and
 * set_solution_theta): a Vec is a pointer to a host array with its length. */
struct RefShimVec { std::vector<double> v; };
typedef RefShimVec *Vec;
typedef int PetscErrorCode;
#define TRYCXX(f) (f)
inline int VecDuplicate(Vec a, Vec *b) { *b = new RefShimVec(); (*b)->v.assign(a->v.size(), 0.0); return 0; }
inline int VecCopy(Vec a, Vec b) { b->v = a->v; return 0; }
inline int VecDestroy(Vec *a) { delete *a; *a = nullptr; return 0; }
inline int VecGetArray(Vec a, double **p) { *p = a->v.data(); return 0; }
inline int VecRestoreArray(Vec, double **p) { *p = nullptr; return 0; }

#include "general/algebra/vector/generalvector.h"
#include "general/common/decomposition.h"
#include "general/data/generaldata.h"

#endif
