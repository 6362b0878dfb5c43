// ref_harness.cpp — a C entry layer over Spira's own templates, so the tests
// can run Spira itself (built from its sources by oracle/Makefile into
// oracle/_ref/libspira_ref.so) on the same inputs as the GPU engine.
//
// TEST INFRASTRUCTURE ONLY; built only where the Spira source tree exists.
// Everything below calls Spira's public API exactly as a Spira user would:
// matrix / parallel_matrix insert + lock + open, load_csr, serial and
// parallel spmv / spgemm / transpose.
#include <spira/parallel/parallel.hpp>
#include <spira/serial/serial.hpp>
#include <spira/spira.hpp>

#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <vector>

namespace {

using SoA = spira::layout::tags::soa_tag;
using AoS = spira::layout::tags::aos_tag;
using MatS = spira::matrix<SoA, uint32_t, double>;
using MatA = spira::matrix<AoS, uint32_t, double>;
using PMatS = spira::parallel::parallel_matrix<SoA, uint32_t, double>;

struct RefCsr {
    uint64_t n_rows, n_cols, nnz, capacity;
    uint64_t *off;
    uint32_t *cols;
    double *vals;
};

thread_local char g_err[512];

int fail(const std::exception &e, int code) {
    std::snprintf(g_err, sizeof(g_err), "%s", e.what());
    return code;
}

template <class Csr>
void export_soa(const Csr &csr, uint64_t n_rows, uint64_t n_cols, RefCsr *out) {
    out->n_rows = n_rows;
    out->n_cols = n_cols;
    out->nnz = csr.nnz;
    out->capacity = csr.capacity;
    out->off = static_cast<uint64_t *>(std::malloc((n_rows + 1) * sizeof(uint64_t)));
    out->cols = static_cast<uint32_t *>(std::malloc((csr.nnz ? csr.nnz : 1) * sizeof(uint32_t)));
    out->vals = static_cast<double *>(std::malloc((csr.nnz ? csr.nnz : 1) * sizeof(double)));
    for (uint64_t i = 0; i <= n_rows; ++i) out->off[i] = csr.offsets[i];
    if (csr.nnz) {
        std::memcpy(out->cols, csr.cols.get(), csr.nnz * sizeof(uint32_t));
        std::memcpy(out->vals, csr.vals.get(), csr.nnz * sizeof(double));
    }
}

template <class Csr>
void export_aos(const Csr &csr, uint64_t n_rows, uint64_t n_cols, RefCsr *out) {
    out->n_rows = n_rows;
    out->n_cols = n_cols;
    out->nnz = csr.nnz;
    out->capacity = csr.capacity;
    out->off = static_cast<uint64_t *>(std::malloc((n_rows + 1) * sizeof(uint64_t)));
    out->cols = static_cast<uint32_t *>(std::malloc((csr.nnz ? csr.nnz : 1) * sizeof(uint32_t)));
    out->vals = static_cast<double *>(std::malloc((csr.nnz ? csr.nnz : 1) * sizeof(double)));
    for (uint64_t i = 0; i <= n_rows; ++i) out->off[i] = csr.offsets[i];
    for (uint64_t k = 0; k < csr.nnz; ++k) {
        out->cols[k] = csr.pairs.get()[k].column;
        out->vals[k] = csr.pairs.get()[k].value;
    }
}

spira::csr_storage<SoA, uint32_t, double> make_storage(const RefCsr *A) {
    spira::csr_storage<SoA, uint32_t, double> s(A->n_rows, A->nnz);
    for (uint64_t i = 0; i <= A->n_rows; ++i) s.offsets[i] = A->off[i];
    if (A->nnz) {
        std::memcpy(s.cols.get(), A->cols, A->nnz * sizeof(uint32_t));
        std::memcpy(s.vals.get(), A->vals, A->nnz * sizeof(double));
    }
    return s;
}

MatS load(const RefCsr *A) {
    MatS m(A->n_rows, A->n_cols);
    m.load_csr(make_storage(A));
    return m;
}

// parallel_matrix: fill every partition from a CSR, lock.
void fill_parallel(PMatS &pm, const RefCsr *A) {
    pm.parallel_fill([A](auto &rows, std::size_t rs, std::size_t re, std::size_t) {
        for (std::size_t r = rs; r < re; ++r)
            for (uint64_t k = A->off[r]; k < A->off[r + 1]; ++k) rows[r - rs].insert(A->cols[k], A->vals[k]);
    });
    pm.lock();
}

void export_parallel(const PMatS &pm, RefCsr *out) {
    const uint64_t n = pm.n_rows();
    out->n_rows = n;
    out->n_cols = pm.n_cols();
    out->off = static_cast<uint64_t *>(std::malloc((n + 1) * sizeof(uint64_t)));
    std::vector<uint32_t> c;
    std::vector<double> v;
    out->off[0] = 0;
    out->capacity = 0;
    for (std::size_t t = 0; t < pm.n_threads(); ++t) {
        const auto &p = pm.partition_at(t);
        for (std::size_t i = 0; i < p.rows.size(); ++i) {
            for (std::size_t k = p.csr.offsets[i]; k < p.csr.offsets[i + 1]; ++k) {
                c.push_back(p.csr.cols.get()[k]);
                v.push_back(p.csr.vals.get()[k]);
            }
            out->off[p.row_start + i + 1] = c.size();
        }
        out->capacity += p.csr.capacity;
    }
    out->nnz = c.size();
    out->cols = static_cast<uint32_t *>(std::malloc((c.size() ? c.size() : 1) * sizeof(uint32_t)));
    out->vals = static_cast<double *>(std::malloc((v.size() ? v.size() : 1) * sizeof(double)));
    if (!c.empty()) {
        std::memcpy(out->cols, c.data(), c.size() * sizeof(uint32_t));
        std::memcpy(out->vals, v.data(), v.size() * sizeof(double));
    }
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g_err; }

void ref_csr_free(RefCsr *A) {
    std::free(A->off);
    std::free(A->cols);
    std::free(A->vals);
    A->off = nullptr;
    A->cols = nullptr;
    A->vals = nullptr;
}

// Insert/lock/open cycles through spira::matrix (layout 0 = AoS, 1 = SoA) or
// parallel_matrix<SoA> (layout 2, n_threads partitions). Epoch e holds
// epoch_len[e] consecutive triples. Returns 0, or 1/2/3 for
// invalid_argument / logic_error / out_of_range.
int ref_lock_epochs(int layout, int n_threads, uint64_t n_rows, uint64_t n_cols, int n_epochs,
                    const uint64_t *epoch_len, const uint32_t *rows, const uint32_t *cols, const double *vals,
                    RefCsr *out) {
    try {
        uint64_t base = 0;
        if (layout == 0 || layout == 1) {
            auto run = [&](auto &m) {
                for (int e = 0; e < n_epochs; ++e) {
                    if (e) m.open();
                    for (uint64_t i = base; i < base + epoch_len[e]; ++i) m.insert(rows[i], cols[i], vals[i]);
                    base += epoch_len[e];
                    m.lock();
                }
            };
            if (layout == 1) {
                MatS m(n_rows, n_cols);
                run(m);
                export_soa(*m.csr(), n_rows, n_cols, out);
            } else {
                MatA m(n_rows, n_cols);
                run(m);
                export_aos(*m.csr(), n_rows, n_cols, out);
            }
        } else {
            PMatS pm(n_rows, n_cols, n_threads);
            for (int e = 0; e < n_epochs; ++e) {
                if (e) pm.open();
                for (uint64_t i = base; i < base + epoch_len[e]; ++i) pm.insert(rows[i], cols[i], vals[i]);
                base += epoch_len[e];
                pm.lock();
            }
            export_parallel(pm, out);
        }
        return 0;
    } catch (const std::out_of_range &e) {
        return fail(e, 3);
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

// mode 0: serial spmv on matrix<SoA,u32,double> (the sparse_dot_double
// overload, serial/spmv.hpp:141-186); mode 1: serial generic loop through an
// AoS matrix (serial/spmv.hpp:56-66); mode 2: parallel spmv on
// parallel_matrix<SoA> with n_threads partitions (the threaded SIMD path).
int ref_spmv(int mode, int n_threads, const RefCsr *A, const double *x, double *y) {
    try {
        std::vector<double> xv(x, x + A->n_cols), yv(A->n_rows, 0.0);
        if (mode == 0) {
            MatS m = load(A);
            spira::serial::algorithms::spmv(m, xv, yv);
        } else if (mode == 1) {
            MatA m(A->n_rows, A->n_cols);
            for (uint64_t r = 0; r < A->n_rows; ++r)
                for (uint64_t k = A->off[r]; k < A->off[r + 1]; ++k) m.insert(r, A->cols[k], A->vals[k]);
            m.lock();
            spira::serial::algorithms::spmv(m, xv, yv);
        } else {
            PMatS pm(A->n_rows, A->n_cols, n_threads);
            fill_parallel(pm, A);
            spira::parallel::algorithms::spmv(pm, xv, yv);
        }
        std::memcpy(y, yv.data(), A->n_rows * sizeof(double));
        return 0;
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

// Times `reps` parallel SpMVs (seconds per call, median-free mean) on a
// parallel_matrix built once: Spira's threaded SIMD CPU path.
double ref_spmv_parallel_time(int n_threads, const RefCsr *A, const double *x, double *y, int reps) {
    PMatS pm(A->n_rows, A->n_cols, n_threads);
    fill_parallel(pm, A);
    std::vector<double> xv(x, x + A->n_cols), yv(A->n_rows, 0.0);
    spira::parallel::algorithms::spmv(pm, xv, yv);
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < reps; ++i) spira::parallel::algorithms::spmv(pm, xv, yv);
    auto t1 = std::chrono::steady_clock::now();
    std::memcpy(y, yv.data(), A->n_rows * sizeof(double));
    return std::chrono::duration<double>(t1 - t0).count() / reps;
}

// C = A * B: serial (parallel == 0) or parallel with n_threads partitions.
int ref_spgemm(int parallel, int n_threads, const RefCsr *A, const RefCsr *B, RefCsr *C) {
    try {
        if (!parallel) {
            MatS a = load(A), b = load(B);
            MatS c = spira::serial::algorithms::spgemm(a, b);
            export_soa(*c.csr(), A->n_rows, B->n_cols, C);
        } else {
            PMatS a(A->n_rows, A->n_cols, n_threads), b(B->n_rows, B->n_cols, n_threads);
            fill_parallel(a, A);
            fill_parallel(b, B);
            PMatS c = spira::parallel::algorithms::spgemm(a, b);
            export_parallel(c, C);
        }
        return 0;
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

int ref_transpose(int parallel, int n_threads, const RefCsr *A, RefCsr *T) {
    try {
        if (!parallel) {
            MatS a = load(A);
            MatS t = spira::serial::algorithms::transpose(a);
            export_soa(*t.csr(), A->n_cols, A->n_rows, T);
        } else {
            PMatS a(A->n_rows, A->n_cols, n_threads);
            fill_parallel(a, A);
            PMatS t = spira::parallel::algorithms::transpose(a);
            export_parallel(t, T);
        }
        return 0;
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

// C = A + B: serial MatrixAddition (parallel == 0) or the parallel one with
// n_threads partitions.
int ref_add(int parallel, int n_threads, const RefCsr *A, const RefCsr *B, RefCsr *C) {
    try {
        if (!parallel) {
            MatS a = load(A), b = load(B);
            MatS c = spira::serial::algorithms::MatrixAddition(a, b);
            export_soa(*c.csr(), A->n_rows, A->n_cols, C);
        } else {
            PMatS a(A->n_rows, A->n_cols, n_threads), b(B->n_rows, B->n_cols, n_threads);
            fill_parallel(a, A);
            fill_parallel(b, B);
            PMatS c = spira::parallel::algorithms::MatrixAddition(a, b);
            export_parallel(c, C);
        }
        return 0;
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

// A * s or A / s: the copy path (in_place == 0: multiplication_scaler(mat,
// out, s)) or the in-place path on the re-opened matrix followed by lock().
// Returns 4 for std::domain_error.
int ref_scale(int in_place, int divide, const RefCsr *A, double s, RefCsr *C) {
    try {
        MatS a = load(A);
        if (in_place) {
            a.open();
            if (divide) spira::serial::algorithms::division_scaler(a, s);
            else spira::serial::algorithms::multiplication_scaler(a, s);
            a.lock();
            export_soa(*a.csr(), A->n_rows, A->n_cols, C);
        } else {
            MatS out(A->n_rows, A->n_cols);
            if (divide) spira::serial::algorithms::division_scaler(a, out, s);
            else spira::serial::algorithms::multiplication_scaler(a, out, s);
            export_soa(*out.csr(), A->n_rows, A->n_cols, C);
        }
        return 0;
    } catch (const std::domain_error &e) {
        return fail(e, 4);
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    } catch (const std::logic_error &e) {
        return fail(e, 2);
    }
}

// accumulate(mat) on a locked matrix: every row's sum.
void ref_row_sums(const RefCsr *A, double *out) {
    MatS a = load(A);
    const std::vector<double> acc = spira::serial::algorithms::accumulate(a);
    std::memcpy(out, acc.data(), A->n_rows * sizeof(double));
}

// compute_partition_boundaries over the CSR's row lengths.
void ref_partition(const RefCsr *A, uint64_t n_parts, uint64_t *bounds) {
    std::vector<std::size_t> row_nnz(A->n_rows);
    for (uint64_t r = 0; r < A->n_rows; ++r) row_nnz[r] = A->off[r + 1] - A->off[r];
    const auto b = spira::parallel::compute_partition_boundaries(row_nnz, n_parts);
    for (uint64_t t = 0; t <= n_parts; ++t) bounds[t] = b[t];
}

// load_csr validation: 0 if Spira accepts the CSR, 1 (invalid_argument) else.
int ref_load_check(const RefCsr *A) {
    try {
        MatS m = load(A);
        (void)m;
        return 0;
    } catch (const std::invalid_argument &e) {
        return fail(e, 1);
    }
}

}  // extern "C"
