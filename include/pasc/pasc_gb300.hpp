// pasc_gb300.hpp -- header-only C++17 class surface over the C ABI of pasc_gb300.h, mirroring
// the classes a PASC_inference driver builds (examples/test_signal1D/test_signal1D.cpp:188-288):
//
//   Decomposition(T, R, K, xdim, DDT_size)          include/general/common/decomposition.h:55
//   Signal1DData(filename) / TSData                 include/general/data/{signal1Ddata,tsdata}.h
//   GraphH1FEMModel(tsdata, epssqr, fem, usethetainpenalty)   include/general/model/graphh1fem.h:75
//   TSSolver(tsdata, annealing)                     include/general/solver/tssolver.h:80-104
//   SPGQPSolver (TSSolver::get_gammasolver())       include/general/solver/spgqpsolver.h:118-151
//
// Options use the reference's console keys (spgqpsolver_maxit, tssolver_eps, ...).  Everything
// computes on the GPU through libpasc_gb300.so; C ABI failures become pasc_gb300::Error
// exceptions (the reference prints and continues, include/external/petscvector/algebra/
// vector/petscvector.h:51).  Also: RAII handles Problem and Batch, PETSc binary vector I/O
// (the format of the reference's data files) and the seeded uniform generator the Python
// package uses for gamma0, so both front ends solve identical inputs.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../pasc_gb300.h"

namespace pasc_gb300 {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &msg)
        : std::runtime_error("pasc_gb300 error " + std::to_string(code) + ": " + msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc)
{
    if (rc != PASC_OK) throw Error(rc, pasc_gb300_last_error());
}

using Options = std::map<std::string, double>;

// ---------------------------------------------------------------------------------------
// seeded uniforms: splitmix64 of (seed, stream, index), the top 53 bits scaled to [0, 1)
// ---------------------------------------------------------------------------------------
inline uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline std::vector<double> uniform(uint64_t seed, uint64_t stream, size_t n)
{
    const uint64_t key = splitmix64(splitmix64(seed) ^ stream);
    std::vector<double> u(n);
    for (size_t i = 0; i < n; i++)
        u[i] = (double)(splitmix64((uint64_t)i * 0x9E3779B97F4A7C15ull + key) >> 11) * (1.0 / 9007199254740992.0);
    return u;
}

// ---------------------------------------------------------------------------------------
// PETSc binary vectors: int32 class id 1211214, int32 length, the values as big-endian FP64
// (the files of examples/test_signal1D/data)
// ---------------------------------------------------------------------------------------
namespace detail {
inline uint32_t be32(const unsigned char *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
inline void put_be32(unsigned char *p, uint32_t v)
{
    p[0] = (unsigned char)(v >> 24); p[1] = (unsigned char)(v >> 16); p[2] = (unsigned char)(v >> 8); p[3] = (unsigned char)v;
}
}  // namespace detail

inline std::vector<double> load_vec(const std::string &path)
{
    std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path.c_str(), "rb"), &std::fclose);
    if (!f) throw Error(PASC_ERR_ARG, "cannot open " + path);
    unsigned char hdr[8];
    if (std::fread(hdr, 1, 8, f.get()) != 8 || detail::be32(hdr) != 1211214u)
        throw Error(PASC_ERR_ARG, path + ": not a PETSc binary vector");
    const uint32_t n = detail::be32(hdr + 4);
    std::vector<unsigned char> raw((size_t)n * 8);
    if (std::fread(raw.data(), 1, raw.size(), f.get()) != raw.size()) throw Error(PASC_ERR_ARG, path + ": truncated");
    std::vector<double> v(n);
    for (uint32_t i = 0; i < n; i++) {
        uint64_t b = 0;
        for (int q = 0; q < 8; q++) b = b << 8 | raw[(size_t)i * 8 + q];
        std::memcpy(&v[i], &b, 8);
    }
    return v;
}

inline void save_vec(const std::string &path, const std::vector<double> &v)
{
    std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path.c_str(), "wb"), &std::fclose);
    if (!f) throw Error(PASC_ERR_ARG, "cannot write " + path);
    std::vector<unsigned char> raw(8 + v.size() * 8);
    detail::put_be32(raw.data(), 1211214u);
    detail::put_be32(raw.data() + 4, (uint32_t)v.size());
    for (size_t i = 0; i < v.size(); i++) {
        uint64_t b;
        std::memcpy(&b, &v[i], 8);
        for (int q = 0; q < 8; q++) raw[8 + i * 8 + q] = (unsigned char)(b >> (56 - 8 * q));
    }
    if (std::fwrite(raw.data(), 1, raw.size(), f.get()) != raw.size()) throw Error(PASC_ERR_ARG, path + ": write failed");
}

// ---------------------------------------------------------------------------------------
// RAII handles
// ---------------------------------------------------------------------------------------
// Page-locked host memory from pasc_gb300_host_alloc (copies at the host link's full rate),
// freed with the object.  The reference's vectors live in PETSc-allocated host arrays.
template <typename V>
class HostBuffer {
public:
    explicit HostBuffer(size_t n) : n_(n)
    {
        void *p = nullptr;
        check(pasc_gb300_host_alloc(&p, (unsigned long)(n * sizeof(V))));
        p_.reset(static_cast<V *>(p));
    }
    V *data() { return p_.get(); }
    const V *data() const { return p_.get(); }
    size_t size() const { return n_; }
    V &operator[](size_t i) { return p_.get()[i]; }

private:
    struct Del {
        void operator()(V *p) const { pasc_gb300_host_free(p); }
    };
    std::unique_ptr<V, Del> p_;
    size_t n_;
};

class Problem {
public:
    Problem(long T, int K, double epssqr, int precision = PASC_PREC_MIXED, int xdim = 1, int device = 0)
        : T_(T), K_(K), xdim_(xdim)
    {
        pasc_gb300_problem *p = nullptr;
        check(pasc_gb300_create(&p, T, K, xdim, precision, epssqr, device));
        h_.reset(p);
    }
    // graph / image mode: T timesteps on a graph of R = nbr_ptr.size() - 1 nodes (CSR lists,
    // sorted, symmetric); the problem holds T*R blocks of K
    Problem(long T, const std::vector<int> &nbr_ptr, const std::vector<int> &nbr_idx, int K, double epssqr,
            int precision = PASC_PREC_MIXED, int device = 0)
        : T_(T * (long)(nbr_ptr.size() - 1)), K_(K), xdim_(1)
    {
        if (nbr_ptr.size() < 2) throw Error(PASC_ERR_ARG, "graph problem: nbr_ptr needs R + 1 >= 2 entries");
        const int one = 0;
        pasc_gb300_problem *p = nullptr;
        check(pasc_gb300_create_graph(&p, T, (long)nbr_ptr.size() - 1, K, precision, epssqr, device, nbr_ptr.data(),
                                      nbr_idx.empty() ? &one : nbr_idx.data()));
        h_.reset(p);
    }
    long T() const { return T_; }
    int K() const { return K_; }
    int xdim() const { return xdim_; }
    pasc_gb300_problem *handle() const { return h_.get(); }

    void set_epssqr(double e, bool scalef = true) { check(pasc_gb300_set_epssqr(h_.get(), e, scalef ? 1 : 0)); }
    void set_data(const std::vector<double> &x) { need(x, (size_t)T_ * xdim_); check(pasc_gb300_set_data(h_.get(), x.data())); }
    void set_gamma(const std::vector<double> &g) { need(g, (size_t)T_ * K_); check(pasc_gb300_set_gamma(h_.get(), g.data())); }
    void set_theta(const std::vector<double> &t) { need(t, (size_t)K_ * xdim_); check(pasc_gb300_set_theta(h_.get(), t.data())); }
    std::vector<double> get_gamma() const
    {
        std::vector<double> g((size_t)T_ * K_);
        check(pasc_gb300_get_gamma(h_.get(), g.data()));
        return g;
    }
    // FP32 host buffers (the mixed path's device format: half the bytes, no conversion)
    void set_data_f32(const float *x, size_t n) { need_n(n, (size_t)T_ * xdim_); check(pasc_gb300_set_data_f32(h_.get(), x)); }
    void set_gamma_f32(const float *g, size_t n) { need_n(n, (size_t)T_ * K_); check(pasc_gb300_set_gamma_f32(h_.get(), g)); }
    void get_gamma_f32(float *g, size_t n) const { need_n(n, (size_t)T_ * K_); check(pasc_gb300_get_gamma_f32(h_.get(), g)); }
    std::vector<double> get_theta() const
    {
        std::vector<double> t((size_t)K_ * xdim_);
        check(pasc_gb300_get_theta(h_.get(), t.data()));
        return t;
    }
    void permute_gamma() { check(pasc_gb300_permute_gamma(h_.get())); }
    void set_fem(double fem_reduce, int fem_type) { check(pasc_gb300_set_fem(h_.get(), fem_reduce, fem_type)); }
    // timesteps of the gamma QP (ceil(T*fem_reduce) under FEM coarsening, else T)
    long get_T_reduced() const
    {
        double r;
        int t;
        long T2;
        check(pasc_gb300_get_fem(h_.get(), &r, &t, &T2));
        return T2;
    }
    // -1: chosen by timing at the first solve; 0: one timestep per thread; 1: bulk-copy tiles
    void set_sweep_variant(int v) { check(pasc_gb300_set_sweep_variant(h_.get(), v)); }
    int get_sweep_variant() const
    {
        int v = -1;
        check(pasc_gb300_get_sweep_variant(h_.get(), &v));
        return v;
    }
    // FP64 Newton rounds on the face the last solve ended on, to the QP optimum (pasc_gb300_polish)
    pasc_gb300_polish_stats polish(int rounds = 4)
    {
        pasc_gb300_polish_opts o;
        pasc_gb300_polish_default_opts(&o);
        o.rounds = rounds;
        pasc_gb300_polish_stats st{};
        check(pasc_gb300_polish(h_.get(), &o, &st));
        return st;
    }
    // 0 automatic (SPGQPSolver), 1 SPGQPSolver, 2 SPGQPSolverC
    void set_gamma_solver_type(int t) { check(pasc_gb300_set_gamma_solver_type(h_.get(), t)); }
    void set_usethetainpenalty(bool on) { check(pasc_gb300_set_usethetainpenalty(h_.get(), on ? 1 : 0)); }
    bool get_usethetainpenalty() const
    {
        int on = 0;
        check(pasc_gb300_get_usethetainpenalty(h_.get(), &on));
        return on != 0;
    }
    void update_theta() { check(pasc_gb300_update_theta(h_.get())); }
    void update_b() { check(pasc_gb300_update_b(h_.get())); }
    pasc_gb300_spgqp_stats spgqp_solve(const pasc_gb300_spgqp_opts &o)
    {
        pasc_gb300_spgqp_stats st;
        check(pasc_gb300_spgqp_solve(h_.get(), &o, &st));
        return st;
    }
    pasc_gb300_ts_stats ts_solve(const pasc_gb300_ts_opts &ts, const pasc_gb300_spgqp_opts &o,
                                 const std::vector<double> *gamma_restart = nullptr)
    {
        pasc_gb300_ts_stats st;
        check(pasc_gb300_ts_solve(h_.get(), &ts, &o, gamma_restart ? gamma_restart->data() : nullptr, &st));
        return st;
    }
    double get_fx() const
    {
        double f;
        check(pasc_gb300_get_fx(h_.get(), &f));
        return f;
    }
    double abserr_reconstructed(const std::vector<double> &solution) const
    {
        need(solution, (size_t)T_);
        double e;
        check(pasc_gb300_abserr_reconstructed(h_.get(), solution.data(), &e));
        return e;
    }
    std::vector<int> argmax_labels() const
    {
        std::vector<int> l((size_t)T_);
        check(pasc_gb300_argmax_labels(h_.get(), l.data()));
        return l;
    }

private:
    struct Del {
        void operator()(pasc_gb300_problem *p) const { pasc_gb300_destroy(p); }
    };
    static void need(const std::vector<double> &v, size_t n) { need_n(v.size(), n); }
    static void need_n(size_t got, size_t n)
    {
        if (got != n) throw Error(PASC_ERR_ARG, "expected " + std::to_string(n) + " values, got " + std::to_string(got));
    }
    std::unique_ptr<pasc_gb300_problem, Del> h_;
    long T_;
    int K_, xdim_;
};

class Batch {
public:
    Batch(const std::vector<long> &T, const std::vector<int> &K, const std::vector<double> &epssqr, int device = 0)
        : T_(T), K_(K)
    {
        if (T.size() != K.size() || T.size() != epssqr.size()) throw Error(PASC_ERR_ARG, "T, K and epssqr sizes differ");
        pasc_gb300_batch *b = nullptr;
        check(pasc_gb300_batch_create(&b, (int)T.size(), T.data(), K.data(), epssqr.data(), device));
        h_.reset(b);
    }
    int size() const { return (int)T_.size(); }
    // one graph launch per solve with the loops decided on the device (default), or host-driven
    void set_loop(bool device_loop, int chunk = 4) { check(pasc_gb300_batch_set_loop(h_.get(), device_loop ? 1 : 0, chunk)); }
    // work items of the batched sweeps: 0 sized from the segments still running, -c with about
    // c items per resident block, 2..64 fixed items of that many tiles
    void set_segment_tiles(int tiles) { check(pasc_gb300_batch_set_segment_tiles(h_.get(), tiles)); }
    int get_segment_tiles() const
    {
        int t = 0;
        check(pasc_gb300_batch_get_segment_tiles(h_.get(), &t, nullptr));
        return t;
    }
    void set_data(int i, const std::vector<double> &x) { check(pasc_gb300_batch_set_data(h_.get(), i, x.data())); }
    void set_gamma(int i, const std::vector<double> &g) { check(pasc_gb300_batch_set_gamma(h_.get(), i, g.data())); }
    void set_theta(int i, const std::vector<double> &t) { check(pasc_gb300_batch_set_theta(h_.get(), i, t.data())); }
    std::vector<double> get_gamma(int i) const
    {
        std::vector<double> g((size_t)T_.at(i) * K_.at(i));
        check(pasc_gb300_batch_get_gamma(h_.get(), i, g.data()));
        return g;
    }
    std::vector<double> get_theta(int i) const
    {
        std::vector<double> t((size_t)K_.at(i));
        check(pasc_gb300_batch_get_theta(h_.get(), i, t.data()));
        return t;
    }
    std::vector<pasc_gb300_ts_stats> ts_solve(const pasc_gb300_ts_opts &ts, const pasc_gb300_spgqp_opts &o)
    {
        std::vector<pasc_gb300_ts_stats> st(T_.size());
        check(pasc_gb300_batch_ts_solve(h_.get(), &ts, &o, st.data()));
        return st;
    }

private:
    struct Del {
        void operator()(pasc_gb300_batch *b) const { pasc_gb300_batch_destroy(b); }
    };
    std::unique_ptr<pasc_gb300_batch, Del> h_;
    std::vector<long> T_;
    std::vector<int> K_;
};

// ---------------------------------------------------------------------------------------
// options by the reference's console keys
// ---------------------------------------------------------------------------------------
inline pasc_gb300_spgqp_opts spgqp_opts_from(const Options &opt)
{
    pasc_gb300_spgqp_opts o;
    pasc_gb300_spgqp_default_opts(&o);
    for (const auto &kv : opt) {
        const std::string &k = kv.first;
        const double v = kv.second;
        if (k == "spgqpsolver_maxit") o.maxit = (int)v;
        else if (k == "spgqpsolver_eps") o.eps = v;
        else if (k == "spgqpsolver_m") o.m = (int)v;
        else if (k == "spgqpsolver_gamma") o.gamma = v;
        else if (k == "spgqpsolver_sigma1") o.sigma1 = v;
        else if (k == "spgqpsolver_sigma2") o.sigma2 = v;
        else if (k == "spgqpsolver_alphainit") o.alphainit = v;
        else if (k == "spgqpsolver_stop_difff") o.stop_difff = (int)v;
        else if (k == "spgqpsolver_stop_normgp") o.stop_normgp = (int)v;
        else if (k == "spgqpsolver_stop_normgp_normb") o.stop_normgp_normb = (int)v;
        else if (k == "spgqpsolver_stop_Anormgp") o.stop_Anormgp = (int)v;
        else if (k == "spgqpsolver_stop_Anormgp_normb") o.stop_Anormgp_normb = (int)v;
    }
    return o;
}

inline pasc_gb300_ts_opts ts_opts_from(const Options &opt)
{
    pasc_gb300_ts_opts o;
    pasc_gb300_ts_default_opts(&o);
    for (const auto &kv : opt) {
        if (kv.first == "tssolver_maxit") o.maxit = (int)kv.second;
        else if (kv.first == "tssolver_eps") o.eps = kv.second;
        else if (kv.first == "tssolver_init_permute") o.init_permute = (int)kv.second;
    }
    return o;
}

// ---------------------------------------------------------------------------------------
// the reference's classes on the path
// ---------------------------------------------------------------------------------------
// BGMGraph<VectorBase> (include/general/algebra/graph/bgmgraph.h): n nodes with coordinates
// (dim values per node, stored dimension by dimension) joined when closer than a threshold
// (process, src/petscvector/algebra/graph/bgmgraph.cpp:73-152); neighbour lists as CSR
// arrays sorted ascending.  BGMGraphGrid1D / BGMGraphGrid2D: the chain and the 4-neighbour
// pixel grid (process_grid).
class BGMGraph {
public:
    BGMGraph() = default;
    BGMGraph(const std::vector<double> &coordinates, int n, int dim) : coords_(coordinates), n_(n), dim_(dim) {}
    BGMGraph(const std::string &filename, int dim = 2) : coords_(load_vec(filename)), dim_(dim)
    {
        n_ = (int)(coords_.size() / (size_t)dim);
    }
    virtual ~BGMGraph() = default;
    void process(double threshold)
    {
        ptr_.assign((size_t)n_ + 1, 0);
        long nnz = 0;
        check(pasc_gb300_graph_threshold(coords_.data(), n_, dim_, threshold, ptr_.data(), nullptr, 0, &nnz));
        idx_.assign((size_t)nnz, 0);
        check(pasc_gb300_graph_threshold(coords_.data(), n_, dim_, threshold, ptr_.data(), idx_.data(), nnz, &nnz));
        threshold_ = threshold;
        processed_ = true;
    }
    int get_n() const { return n_; }
    int get_m() const { return processed_ ? ptr_.back() / 2 : 0; }
    int get_m_max() const
    {
        int m = 0;
        for (int i = 0; i < n_ && processed_; i++) m = std::max(m, ptr_[i + 1] - ptr_[i]);
        return m;
    }
    int get_dim() const { return dim_; }
    double get_threshold() const { return threshold_; }
    bool is_processed() const { return processed_; }
    const std::vector<int> &nbr_ptr() const { return ptr_; }
    const std::vector<int> &nbr_idx() const { return idx_; }
    virtual std::string get_name() const { return "BGMGraph"; }

protected:
    std::vector<double> coords_;
    int n_ = 0, dim_ = 1;
    double threshold_ = -1.0;
    bool processed_ = false;
    std::vector<int> ptr_, idx_;
};

class BGMGraphGrid1D : public BGMGraph {
public:
    explicit BGMGraphGrid1D(int width) : width_(width)
    {
        n_ = width;
        dim_ = 1;
    }
    void process_grid()
    {
        ptr_.assign((size_t)width_ + 1, 0);
        idx_.assign((size_t)std::max(2 * (width_ - 1), 1), 0);
        check(pasc_gb300_graph_grid1d(width_, ptr_.data(), idx_.data()));
        idx_.resize((size_t)ptr_.back());
        threshold_ = 1.1;
        processed_ = true;
    }
    std::string get_name() const override { return "BGMGraphGrid1D"; }

private:
    int width_;
};

class BGMGraphGrid2D : public BGMGraph {
public:
    BGMGraphGrid2D(int width, int height) : width_(width), height_(height)
    {
        n_ = width * height;
        dim_ = 2;
    }
    void process_grid()
    {
        ptr_.assign((size_t)n_ + 1, 0);
        idx_.assign((size_t)std::max(2 * (height_ * (width_ - 1) + width_ * (height_ - 1)), 1), 0);
        check(pasc_gb300_graph_grid2d(width_, height_, ptr_.data(), idx_.data()));
        idx_.resize((size_t)ptr_.back());
        threshold_ = 1.1;
        processed_ = true;
    }
    int get_width() const { return width_; }
    int get_height() const { return height_; }
    std::string get_name() const override { return "BGMGraphGrid2D"; }

private:
    int width_, height_;
};

class Decomposition {
public:
    // Decomposition<VectorBase>(T, R, K, xdim, DDT_size): one GPU; R > 1 nodes without a graph
    // are disjoint (the graph GraphH1FEMModel builds when none is given, graphh1fem.cpp:30-45)
    Decomposition(long T, int R, int K, int xdim = 1, int DDT_size = 1) : T_(T), R_(R), K_(K), xdim_(xdim)
    {
        if (DDT_size != 1) throw Error(PASC_ERR_NOTSUPP, "one GPU per problem: DDT_size must be 1");
        if (R < 1) throw Error(PASC_ERR_ARG, "R must be >= 1");
        if (R > 1) {
            std::vector<double> c((size_t)R);
            for (int r = 0; r < R; r++) c[r] = r;
            auto g = std::make_shared<BGMGraph>(c, R, 1);
            g->process(0.0);
            graph_ = g;
            if (xdim != 1) throw Error(PASC_ERR_NOTSUPP, "graph problems take scalar data (xdim 1)");
        }
    }
    // Decomposition<VectorBase>(T, graph, K, xdim, DDR_size)
    Decomposition(long T, const BGMGraph &graph, int K, int xdim = 1, int DDR_size = 1)
        : T_(T), R_(graph.get_n()), K_(K), xdim_(xdim), graph_(std::make_shared<BGMGraph>(graph))
    {
        if (DDR_size != 1) throw Error(PASC_ERR_NOTSUPP, "one GPU per problem: DDR_size must be 1");
        if (!graph.is_processed()) throw Error(PASC_ERR_STATE, "the graph is not processed");
        if (xdim != 1) throw Error(PASC_ERR_NOTSUPP, "graph problems take scalar data (xdim 1)");
    }
    long get_T() const { return T_; }
    int get_R() const { return R_; }
    int get_K() const { return K_; }
    int get_xdim() const { return xdim_; }
    const BGMGraph *get_graph() const { return graph_.get(); }
    // permute_TRK: blocked k*R*T + r*T + t <-> interleaved (t*R + r)*K + k
    std::vector<double> permute_TRK(const std::vector<double> &v, bool invert = false) const
    {
        std::vector<double> out(v.size());
        for (int k = 0; k < K_; k++)
            for (long r = 0; r < R_; r++)
                for (long t = 0; t < T_; t++) {
                    const size_t b = (size_t)k * R_ * T_ + (size_t)r * T_ + t, i = ((size_t)t * R_ + r) * K_ + k;
                    if (invert) out[b] = v[i];
                    else out[i] = v[b];
                }
        return out;
    }
    // permute_TRxdim: data r*T + t (file order) <-> t*R + r
    std::vector<double> permute_TRxdim(const std::vector<double> &v, bool invert = false) const
    {
        std::vector<double> out(v.size());
        for (long r = 0; r < R_; r++)
            for (long t = 0; t < T_; t++) {
                if (invert) out[(size_t)r * T_ + t] = v[(size_t)t * R_ + r];
                else out[(size_t)t * R_ + r] = v[(size_t)r * T_ + t];
            }
        return out;
    }

private:
    long T_;
    int R_, K_, xdim_;
    std::shared_ptr<BGMGraph> graph_;
};

// Fem<VectorBase>(fem_reduce) (FEM-SUM, include/general/common/fem.h) and FemHat (FEM-HAT,
// include/general/common/femhat.h): temporal coarsening of the gamma step, fem_reduce < 1
class Fem {
public:
    explicit Fem(double fem_reduce = 1.0) : fem_reduce_(fem_reduce) {}
    virtual ~Fem() = default;
    double get_fem_reduce() const { return fem_reduce_; }
    bool is_reduced() const { return fem_reduce_ < 1.0; }
    virtual int type() const { return 0; }
    virtual std::string get_name() const { return "FEM-SUM"; }

private:
    double fem_reduce_;
};

class FemHat : public Fem {
public:
    explicit FemHat(double fem_reduce = 1.0) : Fem(fem_reduce) {}
    int type() const override { return 1; }
    std::string get_name() const override { return "FEM-HAT"; }
};

class GraphH1FEMModel;

class TSData {
public:
    TSData() = default;
    explicit TSData(const std::vector<double> &data) : data_(data) {}
    void set_decomposition(const Decomposition &d) { decomposition_ = std::make_shared<Decomposition>(d); }
    const Decomposition &get_decomposition() const
    {
        if (!decomposition_) throw Error(PASC_ERR_STATE, "TSData: no decomposition set");
        return *decomposition_;
    }
    long get_T() const { return get_decomposition().get_T(); }
    int get_R() const { return get_decomposition().get_R(); }
    int get_K() const { return get_decomposition().get_K(); }
    int get_xdim() const { return get_decomposition().get_xdim(); }
    const std::vector<double> &get_datavector() const { return data_; }
    inline std::vector<double> get_gammavector() const;
    inline std::vector<double> get_thetavector() const;
    double get_aic() const { return aic_; }
    void set_aic(double a) { aic_ = a; }
    void set_model(GraphH1FEMModel *m) { model_ = m; }
    GraphH1FEMModel *get_model() const { return model_; }
    // TSData::load_gammavector: gamma0 in the blocked layout the reference writes, permuted
    inline void load_gammavector(const std::vector<double> &gamma0);
    // hard assignment gamma_tk = [k = argmax] (true argmax; the reference's cutgamma seeds its
    // running maximum with the wrong entry, src/petscvector/data/tsdata.cpp:212)
    inline void cutgamma();
    // data preprocessing (src/petscvector/data/tsdata.cpp:384-560): clamp to [a, b], shift,
    // map [scale_min, scale_max] (default: the data's range) linearly onto [a, b] and back
    // (theta with it); a model's copy of the data is refreshed
    inline void cutdata(double a, double b);
    inline void shiftdata(double a);
    inline void scaledata(double a, double b);
    inline void scaledata(double a, double b, double scale_min, double scale_max);
    inline void unscaledata(double a, double b);

protected:
    inline void data_changed();
    std::vector<double> data_;
    std::shared_ptr<Decomposition> decomposition_;
    GraphH1FEMModel *model_ = nullptr;
    double aic_ = std::numeric_limits<double>::max();
    double scale_min_ = 0.0, scale_max_ = 1.0;
};

class Signal1DData : public TSData {
public:
    explicit Signal1DData(const std::string &filename) : TSData(load_vec(filename)) {}
    explicit Signal1DData(const std::vector<double> &data) : TSData(data) {}
    long get_Tpreliminary() const { return (long)data_.size(); }
    inline double compute_abserr_reconstructed(const std::vector<double> &solution) const;
    // saveSignal1D: <prefix>_gamma.bin (blocked layout) and <prefix>_recovered.bin
    inline void saveSignal1D(const std::string &prefix) const;
};

// ImageData<VectorBase>(decomposition, filename, width, height) (src/petscvector/data/
// imagedata.cpp:7-38): pixels node-major in the file (r*T + t), interleaved here (t*R + r)
class ImageData : public TSData {
public:
    ImageData(const Decomposition &dec, const std::string &filename, int width, int height)
        : ImageData(dec, load_vec(filename), width, height)
    {
    }
    ImageData(const Decomposition &dec, const std::vector<double> &raw, int width, int height)
        : width_(width), height_(height)
    {
        if ((long)raw.size() != dec.get_T() * dec.get_R())
            throw Error(PASC_ERR_ARG, "ImageData: the data does not have T*width*height values");
        set_decomposition(dec);
        data_ = dec.permute_TRxdim(raw);
    }
    int get_width() const { return width_; }
    int get_height() const { return height_; }
    // saveImage (imagedata.cpp:40-103): <prefix>_original.bin, _gamma.bin (blocked),
    // _recovered.bin (sum_k theta_k gamma_k), node-major
    inline void saveImage(const std::string &prefix, bool save_original = true) const;

private:
    int width_, height_;
};

class GraphH1FEMModel {
public:
    // GraphH1FEMModel<VectorBase>(tsdata, epssqr, fem, usethetainpenalty): creates the GPU
    // problem with gamma0 = uniform [0, 1) values (seed, stream 0) in the blocked layout, as
    // set_random leaves it
    GraphH1FEMModel(TSData &tsdata, double epssqr, const Fem *fem = nullptr, bool usethetainpenalty = false,
                    int precision = PASC_PREC_MIXED, uint64_t seed = 13, int device = 0)
        : tsdata_(tsdata), epssqr_(epssqr), usethetainpenalty_(usethetainpenalty),
          fem_reduce_(fem ? fem->get_fem_reduce() : 1.0), problem_(make_problem(tsdata, epssqr, precision, device))
    {
        const long T = tsdata.get_T() * tsdata.get_R();  // blocks of K
        const int K = tsdata.get_K();
        if (fem && fem->is_reduced()) problem_.set_fem(fem->get_fem_reduce(), fem->type());
        if (usethetainpenalty) problem_.set_usethetainpenalty(true);
        problem_.set_data(tsdata.get_datavector());
        problem_.set_gamma(uniform(seed, 0, (size_t)T * K));
        problem_.set_theta(std::vector<double>((size_t)K * tsdata.get_xdim(), 0.0));
        tsdata.set_model(this);
    }
    void set_epssqr(double e)
    {
        epssqr_ = e;
        problem_.set_epssqr(e);
    }
    double get_epssqr() const { return epssqr_; }
    double get_aic(double L) const { return 2.0 * std::log(L) + tsdata_.get_K(); }
    bool get_usethetainpenalty() const { return usethetainpenalty_; }
    std::string get_name() const { return "Graph-H1-FEM Time-Series Model"; }
    // GraphH1FEMModel::get_T / get_T_reduced / get_fem_reduce (graphh1fem.h:456-468)
    long get_T() const { return tsdata_.get_T(); }
    long get_T_reduced() const { return fem_reduce_ < 1.0 ? problem_.get_T_reduced() : tsdata_.get_T(); }
    double get_fem_reduce() const { return fem_reduce_; }
    const BGMGraph *get_graph() const { return tsdata_.get_decomposition().get_graph(); }
    // GraphH1FEMModel::get_L: the gamma QP's objective at the current gamma and theta
    // (graphh1fem.h:366-370)
    double get_L() const { return problem_.get_fx(); }
    // GraphH1FEMModel::get_linear_quadratic sets both terms to 0 (graphh1fem.h:373-377)
    void get_linear_quadratic(double *linearL, double *quadraticL) const
    {
        *linearL = 0.0;
        *quadraticL = 0.0;
    }
    Problem &problem() { return problem_; }
    const Problem &problem() const { return problem_; }

private:
    static Problem make_problem(const TSData &d, double epssqr, int precision, int device)
    {
        const BGMGraph *g = d.get_decomposition().get_graph();
        if (g) return Problem(d.get_T(), g->nbr_ptr(), g->nbr_idx(), d.get_K(), epssqr, precision, device);
        return Problem(d.get_T(), d.get_K(), epssqr, precision, d.get_xdim(), device);
    }
    TSData &tsdata_;
    double epssqr_;
    bool usethetainpenalty_;
    double fem_reduce_;
    Problem problem_;
};

inline std::vector<double> TSData::get_gammavector() const
{
    if (!model_) throw Error(PASC_ERR_STATE, "TSData: no model");
    return model_->problem().get_gamma();
}
inline std::vector<double> TSData::get_thetavector() const
{
    if (!model_) throw Error(PASC_ERR_STATE, "TSData: no model");
    return model_->problem().get_theta();
}
inline void TSData::load_gammavector(const std::vector<double> &gamma0)
{
    if (!model_) throw Error(PASC_ERR_STATE, "TSData: no model");
    model_->problem().set_gamma(gamma0);
    model_->problem().permute_gamma();
}
inline void TSData::data_changed()
{
    if (model_) model_->problem().set_data(data_);
}
inline void TSData::cutdata(double a, double b)
{
    for (double &v : data_) v = v > b ? b : (v < a ? a : v);
    data_changed();
}
inline void TSData::shiftdata(double a)
{
    for (double &v : data_) v += a;
    data_changed();
}
inline void TSData::scaledata(double a, double b)
{
    if (data_.empty()) return;
    const auto mm = std::minmax_element(data_.begin(), data_.end());
    scaledata(a, b, *mm.first, *mm.second);
}
inline void TSData::scaledata(double a, double b, double scale_min, double scale_max)
{
    scale_min_ = scale_min;
    scale_max_ = scale_max;
    const double k = (b - a) / (scale_max - scale_min), q = a - k * scale_min;
    for (double &v : data_) v = v * k + q;
    data_changed();
    if (model_) {
        std::vector<double> th = model_->problem().get_theta();
        for (double &t : th) t = k * t + q;
        model_->problem().set_theta(th);
    }
}
inline void TSData::unscaledata(double a, double b)
{
    const double k = (b - a) / (scale_max_ - scale_min_), q = a - k * scale_min_;
    for (double &v : data_) v = (v - q) * (1.0 / k);
    data_changed();
    if (model_) {
        std::vector<double> th = model_->problem().get_theta();
        for (double &t : th) t = (t - q) / k;
        model_->problem().set_theta(th);
    }
}
inline void TSData::cutgamma()
{
    if (!model_) throw Error(PASC_ERR_STATE, "TSData: no model");
    const std::vector<int> lab = model_->problem().argmax_labels();
    const long T = get_T() * get_R();  // blocks of K
    const int K = get_K();
    std::vector<double> g((size_t)T * K, 0.0);
    for (long t = 0; t < T; t++) g[(size_t)t * K + lab[t]] = 1.0;
    model_->problem().set_gamma(g);
}
inline double Signal1DData::compute_abserr_reconstructed(const std::vector<double> &solution) const
{
    if (!model_) throw Error(PASC_ERR_STATE, "Signal1DData: no model");
    return model_->problem().abserr_reconstructed(solution);
}
inline void Signal1DData::saveSignal1D(const std::string &prefix) const
{
    const long T = get_T();
    const int K = get_K();
    const std::vector<double> g = get_gammavector(), th = get_thetavector();
    std::vector<double> blocked((size_t)T * K), rec((size_t)T, 0.0);
    for (long t = 0; t < T; t++)
        for (int k = 0; k < K; k++) {
            blocked[(size_t)k * T + t] = g[(size_t)t * K + k];
            rec[t] += g[(size_t)t * K + k] * th[k];
        }
    save_vec(prefix + "_gamma.bin", blocked);
    save_vec(prefix + "_recovered.bin", rec);
}

inline void ImageData::saveImage(const std::string &prefix, bool save_original) const
{
    const Decomposition &dec = get_decomposition();
    if (save_original) save_vec(prefix + "_original.bin", dec.permute_TRxdim(data_, true));
    const std::vector<double> g = get_gammavector(), th = get_thetavector();
    const int K = get_K();
    std::vector<double> rec(data_.size(), 0.0);
    for (size_t s = 0; s < rec.size(); s++)
        for (int k = 0; k < K; k++) rec[s] += g[s * K + k] * th[k];
    save_vec(prefix + "_gamma.bin", dec.permute_TRK(g, true));
    save_vec(prefix + "_recovered.bin", dec.permute_TRxdim(rec, true));
}

class SPGQPSolver {
public:
    SPGQPSolver(GraphH1FEMModel &model, const Options &opt = {}) : model_(model), o_(spgqp_opts_from(opt)) {}
    void solve()
    {
        last_ = model_.problem().spgqp_solve(o_);
        it_sum_ += last_.it;
        hessmult_sum_ += last_.hessmult;
    }
    double get_fx() const { return model_.problem().get_fx(); }
    int get_it() const { return it_sum_; }
    int get_hessmult() const { return hessmult_sum_; }
    const pasc_gb300_spgqp_opts &opts() const { return o_; }
    void add_it(int n) { it_sum_ += n; }

private:
    GraphH1FEMModel &model_;
    pasc_gb300_spgqp_opts o_;
    pasc_gb300_spgqp_stats last_{};
    int it_sum_ = 0, hessmult_sum_ = 0;
};

class TSSolver {
public:
    TSSolver(TSData &tsdata, int annealing = 1, const Options &opt = {})
        : tsdata_(tsdata), annealing_(annealing), opt_(opt), gammasolver_(model(tsdata), opt) {}
    void set_solution_theta(const std::vector<double> &theta)
    {
        model(tsdata_).problem().set_theta(theta);
        thetasolved_ = true;
    }
    void set_annealing(int a) { annealing_ = a; }
    pasc_gb300_ts_stats solve(const std::vector<double> *gamma_restart = nullptr)
    {
        pasc_gb300_ts_opts ts = ts_opts_from(opt_);
        ts.annealing = annealing_;
        ts.thetasolved = thetasolved_ ? 1 : 0;
        stats_ = model(tsdata_).problem().ts_solve(ts, gammasolver_.opts(), gamma_restart);
        L_ = stats_.L;
        gammasolver_.add_it(stats_.spg_it_sum);
        tsdata_.set_aic(stats_.aic);
        return stats_;
    }
    double get_L() const { return L_; }
    SPGQPSolver &get_gammasolver() { return gammasolver_; }
    const pasc_gb300_ts_stats &stats() const { return stats_; }

private:
    static GraphH1FEMModel &model(TSData &d)
    {
        if (!d.get_model()) throw Error(PASC_ERR_STATE, "TSSolver: the data has no model");
        return *d.get_model();
    }
    TSData &tsdata_;
    int annealing_;
    Options opt_;
    SPGQPSolver gammasolver_;
    bool thetasolved_ = false;
    double L_ = std::numeric_limits<double>::max();
    pasc_gb300_ts_stats stats_{};
};

}  // namespace pasc_gb300
