// Eigenvalues and eigenvectors of a symmetric tridiagonal matrix, on the host.
//
// The GPU eigensolver (eigh.cu) reduces the Fock matrix to tridiagonal form T;
// this file finishes the problem in O(n^2) work:
//   * T is split where an off-diagonal element is negligible (|e_i| <= eps ||T||),
//   * the eigenvalues of each unreduced block come from the implicit QL
//     iteration with Wilkinson shifts (EISPACK tql1; Golub & Van Loan, 8.3),
//   * each eigenvector from inverse iteration on T - lambda I with a pivoted LU
//     factorisation, eigenvalues closer than 1e-3 ||T|| forming a cluster whose
//     vectors are orthogonalised against each other by modified Gram-Schmidt
//     (the strategy of LAPACK's dstein).
// Clusters are independent, so their vectors are computed by a small pool of
// host threads; only the ncol lowest eigenvectors are formed when fewer are
// asked for (an SCF iteration needs the occupied ones only).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "internal.h"

namespace hfgpu {

namespace {

constexpr double kEps = 2.220446049250313e-16;

// eigenvalues of the unreduced block (d[0..nb), e[0..nb-1)), in place in d (unsorted)
void ql_eigenvalues(int nb, double* d, double* e)
{
    // e[nb - 1] is used as scratch by the iteration
    for (int l = 0; l < nb; ++l) {
        int iter = 0;
        for (;;) {
            int m = l;
            for (; m < nb - 1; ++m) {
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= kEps * dd) break;
            }
            if (m == l) break;
            HF_CHECK(++iter <= 60, HFGPU_ERR_LINALG, "tridiagonal QL iteration did not converge");
            // Wilkinson shift from the leading 2 x 2 block
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::sqrt(g * g + 1.0);  // values are Fock-matrix sized: no overflow guard
            g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            bool deflated = false;
            for (int i = m - 1; i >= l; --i) {
                const double f = s * e[i], b = c * e[i];
                r = std::sqrt(f * f + g * g);
                e[i + 1] = r;
                if (r == 0.0) {  // the chase met an exact zero: T splits here
                    d[i + 1] -= p;
                    e[m] = 0.0;
                    deflated = true;
                    break;
                }
                const double ri = 1.0 / r;  // one division for both rotation entries
                s = f * ri;
                c = g * ri;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
            }
            if (deflated) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
}

// P (T - x I) = L U for the tridiagonal block, U with two superdiagonals
struct TriLU {
    std::vector<double> u0, u1, u2, l, r0;  // r0 = 1 / u0
    std::vector<char> sw;
    explicit TriLU(int nb) : u0(nb), u1(nb), u2(nb), l(nb), r0(nb), sw(nb) {}
    void factor(int nb, const double* d, const double* e, double x, double tiny)
    {
        auto floor_pivot = [&](double v) { return std::fabs(v) < tiny ? (v < 0 ? -tiny : tiny) : v; };
        // active row: entries in columns (i, i + 1)
        double ad = d[0] - x, as = nb > 1 ? e[0] : 0.0;
        for (int i = 0; i < nb - 1; ++i) {
            const double sub = e[i], nd = d[i + 1] - x, ns = i + 1 < nb - 1 ? e[i + 1] : 0.0;
            if (std::fabs(ad) >= std::fabs(sub)) {
                const double piv = floor_pivot(ad);
                sw[i] = 0;
                u0[i] = piv;
                u1[i] = as;
                u2[i] = 0.0;
                l[i] = sub / piv;
                ad = nd - l[i] * as;
                as = ns;
            } else {
                sw[i] = 1;
                u0[i] = sub;
                u1[i] = nd;
                u2[i] = ns;
                l[i] = ad / sub;
                ad = as - l[i] * nd;
                as = -l[i] * ns;
            }
        }
        u0[nb - 1] = floor_pivot(ad);
        for (int i = 0; i < nb; ++i) r0[i] = 1.0 / u0[i];
    }
    void solve(int nb, double* y) const
    {
        double r = y[0];
        for (int i = 0; i < nb - 1; ++i) {
            if (!sw[i]) {
                y[i] = r;
                r = y[i + 1] - l[i] * r;
            } else {
                const double t = y[i + 1];
                y[i] = t;
                r -= l[i] * t;
            }
        }
        y[nb - 1] = r * r0[nb - 1];
        if (nb >= 2) y[nb - 2] = (y[nb - 2] - u1[nb - 2] * y[nb - 1]) * r0[nb - 2];
        for (int i = nb - 3; i >= 0; --i) y[i] = (y[i] - u1[i] * y[i + 1] - u2[i] * y[i + 2]) * r0[i];
    }
};

void normalize(int nb, double* y)
{
    double s = 0.0;
    for (int i = 0; i < nb; ++i) s += y[i] * y[i];
    s = 1.0 / std::sqrt(s);
    for (int i = 0; i < nb; ++i) y[i] *= s;
}

// y -= sum_k (z_k . y) z_k over the columns c0 .. c1 - 1 of Z (leading dimension ld)
void orthogonalize(int nb, double* y, const double* Z, int ld, int c0, int c1)
{
    for (int k = c0; k < c1; ++k) {
        const double* z = Z + (size_t)k * ld;
        double s = 0.0;
        for (int i = 0; i < nb; ++i) s += z[i] * y[i];
        for (int i = 0; i < nb; ++i) y[i] -= s * z[i];
    }
}

double block_norm(int nb, const double* d, const double* e)
{
    double t = 0.0;
    for (int i = 0; i < nb; ++i)
        t = std::max(t, std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < nb - 1 ? std::fabs(e[i]) : 0.0));
    return t == 0.0 ? 1.0 : t;
}

// eigenvectors j = c0 .. c1 - 1 of one unreduced block (ascending eigenvalues
// lam, one cluster), into columns of Zb (leading dimension nb); each one is
// kept orthogonal to the cluster's earlier vectors
void cluster_vectors(int nb, const double* d, const double* e, const double* lam, int c0, int c1, double tnorm,
                     double* Zb)
{
    const double pert = 10.0 * kEps * tnorm, tiny = kEps * tnorm;
    TriLU lu(nb);
    std::vector<double> y(nb);
    double xprev = 0.0;
    for (int j = c0; j < c1; ++j) {
        double x = lam[j];
        if (j > c0 && x - xprev < pert) x = xprev + pert;  // keep equal eigenvalues apart
        xprev = x;
        lu.factor(nb, d, e, x, tiny);
        uint64_t seed = 0x243F6A8885A308D3ull ^ ((uint64_t)j * 0x9E3779B97F4A7C15ull);
        for (int i = 0; i < nb; ++i) {  // start vector: uniform in (-1, 1), a function of j only
            seed = seed * 6364136223846793005ull + 1442695040888963407ull;
            y[i] = (double)(seed >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
        for (int it = 0; it < 3; ++it) {
            orthogonalize(nb, y.data(), Zb, nb, c0, j);
            normalize(nb, y.data());
            lu.solve(nb, y.data());
        }
        for (int pass = 0; pass < 2; ++pass) orthogonalize(nb, y.data(), Zb, nb, c0, j);
        normalize(nb, y.data());
        std::copy(y.begin(), y.end(), Zb + (size_t)j * nb);
    }
}

// A few persistent worker threads; run(n, f) calls f(0 .. n-1) on them and on
// the calling thread and returns when all are done.  Several host threads may
// call run at once (batched molecules); their jobs are served in order.
class HostPool {
public:
    static HostPool& get()
    {
        static HostPool* pool = new HostPool();  // never destroyed: workers outlive static destructors
        return *pool;
    }
    void run(int ntask, const std::function<void(int)>& f)
    {
        if (ntask <= 0) return;
        if (ntask == 1 || workers_.empty()) {
            for (int i = 0; i < ntask; ++i) f(i);
            return;
        }
        auto job = std::make_shared<Job>();
        job->f = &f;
        job->n = ntask;
        {
            std::lock_guard<std::mutex> lk(m_);
            queue_.push_back(job);
        }
        cv_.notify_all();
        job->work();
        {
            std::unique_lock<std::mutex> lk(job->m);
            job->cv.wait(lk, [&] { return job->done == job->n; });
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            queue_.erase(std::remove(queue_.begin(), queue_.end(), job), queue_.end());
        }
        if (job->err) std::rethrow_exception(job->err);
    }

private:
    struct Job {
        const std::function<void(int)>* f = nullptr;
        int n = 0;
        std::atomic<int> next{0};
        std::mutex m;
        std::condition_variable cv;
        int done = 0;
        std::exception_ptr err;
        void work()
        {
            for (int i; (i = next.fetch_add(1)) < n;) {
                std::exception_ptr e;
                try {
                    (*f)(i);
                } catch (...) {
                    e = std::current_exception();
                }
                std::lock_guard<std::mutex> lk(m);
                if (e && !err) err = e;
                if (++done == n) cv.notify_all();
            }
        }
    };
    HostPool()
    {
        const unsigned hw = std::thread::hardware_concurrency();
        const int nw = (int)std::min(7u, hw > 1 ? hw - 1 : 0u);
        for (int i = 0; i < nw; ++i) workers_.emplace_back([this] { loop(); });
        for (auto& t : workers_) t.detach();
    }
    void loop()
    {
        for (;;) {
            std::shared_ptr<Job> job;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] {
                    for (auto& j : queue_)
                        if (j->next.load() < j->n) return true;
                    return false;
                });
                for (auto& j : queue_)
                    if (j->next.load() < j->n) {
                        job = j;
                        break;
                    }
            }
            if (job) job->work();
        }
    }
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<std::shared_ptr<Job>> queue_;
    std::vector<std::thread> workers_;
};

}  // namespace

void tridiag_eigen(int n, const double* d_in, const double* e_in, double* lam, double* Z, int ncol)
{
    if (n <= 0) return;
    if (ncol < 0 || ncol > n) ncol = n;
    const double split = kEps * block_norm(n, d_in, e_in);
    struct Block {
        int lo, nb, nvec;
        std::vector<double> d, e, w, Z;  // w: ascending eigenvalues; Z: nb x nvec, column-major
        double tnorm;
    };
    std::vector<Block> blocks;
    for (int lo = 0; lo < n;) {
        int hi = lo;
        while (hi < n - 1 && std::fabs(e_in[hi]) > split) ++hi;
        Block b;
        b.lo = lo;
        b.nb = hi - lo + 1;
        b.d.assign(d_in + lo, d_in + lo + b.nb);
        b.e.assign(b.nb, 0.0);
        for (int i = 0; i < b.nb - 1; ++i) b.e[i] = e_in[lo + i];
        b.w = b.d;
        std::vector<double> ew(b.e);
        ql_eigenvalues(b.nb, b.w.data(), ew.data());
        std::sort(b.w.begin(), b.w.end());
        b.tnorm = block_norm(b.nb, b.d.data(), b.e.data());
        blocks.push_back(std::move(b));
        lo = hi + 1;
    }
    // global order of all eigenvalues; vectors only for the ncol lowest
    struct Ev {
        double v;
        int block, j;
    };
    std::vector<Ev> all;
    all.reserve(n);
    for (int b = 0; b < (int)blocks.size(); ++b)
        for (int j = 0; j < blocks[b].nb; ++j) all.push_back({blocks[b].w[j], b, j});
    std::stable_sort(all.begin(), all.end(), [](const Ev& a, const Ev& b) { return a.v < b.v; });
    for (auto& b : blocks) b.nvec = 0;
    for (int k = 0; k < ncol; ++k) {
        Block& b = blocks[all[k].block];
        b.nvec = std::max(b.nvec, all[k].j + 1);
    }
    // one task per cluster (eigenvalues chained by gaps <= 1e-3 ||T_block||)
    struct Task {
        int block, c0, c1;
    };
    std::vector<Task> tasks;
    for (int b = 0; b < (int)blocks.size(); ++b) {
        Block& blk = blocks[b];
        blk.Z.assign((size_t)blk.nb * blk.nvec, 0.0);
        if (blk.nb == 1) {
            if (blk.nvec) blk.Z[0] = 1.0;
            continue;
        }
        const double ortol = 1e-3 * blk.tnorm;
        for (int c0 = 0; c0 < blk.nvec;) {
            int c1 = c0 + 1;
            while (c1 < blk.nvec && blk.w[c1] - blk.w[c1 - 1] <= ortol) ++c1;
            tasks.push_back({b, c0, c1});
            c0 = c1;
        }
    }
    // largest clusters first
    std::stable_sort(tasks.begin(), tasks.end(), [](const Task& a, const Task& b) { return a.c1 - a.c0 > b.c1 - b.c0; });
    const std::function<void(int)> fn = [&](int t) {
        const Task& tk = tasks[t];
        Block& b = blocks[tk.block];
        cluster_vectors(b.nb, b.d.data(), b.e.data(), b.w.data(), tk.c0, tk.c1, b.tnorm, b.Z.data());
    };
    if (tasks.size() >= 4 && n >= 64) HostPool::get().run((int)tasks.size(), fn);
    else for (int t = 0; t < (int)tasks.size(); ++t) fn(t);
    for (int k = 0; k < n; ++k) lam[k] = all[k].v;
    std::fill(Z, Z + (size_t)n * ncol, 0.0);
    for (int k = 0; k < ncol; ++k) {
        const Block& b = blocks[all[k].block];
        const double* z = b.Z.data() + (size_t)all[k].j * b.nb;
        std::copy(z, z + b.nb, Z + (size_t)k * n + b.lo);
    }
}

}  // namespace hfgpu
