// spira_gb300/spira.hpp — C++23 drop-in facade for Spira's sparse hot path,
// backed by the GB300 engine (libspg.so, include/spg.h).
//
// Spira user code keeps its spelling: spira::matrix<Layout, I, V, ...> with
// insert / lock / open / get / contains / nnz / row_nnz / csr / load_csr and the
// operators A*x, A*B, ~A (matrix.hpp:22-180, matrix_operators.hpp:67-150);
// spira::serial::algorithms::{spmv, spgemm, transpose, transpose_itself}
// (serial/*.hpp); spira::parallel::parallel_matrix with insert / parallel_fill
// / lock / open / rebalance / partition_at / execute and
// spira::parallel::algorithms::{spmv, spgemm, transpose}
// (parallel/parallel_matrix.hpp:51-267, parallel/algorithms/*.hpp).
//
// The matrix lives on the GPU as one CSR (uint64 offsets, uint32 columns,
// FP64 values). Open-mode inserts are staged on the host in insertion order
// and merged on the device by lock(). Status codes of the C ABI come back as
// Spira's exception types: std::invalid_argument, std::logic_error,
// std::out_of_range, std::bad_alloc, std::runtime_error (CUDA).
// GPU execution covers I = uint32_t, V = double (Spira's SIMD fast-path
// types); other instantiations are rejected at compile time. There is no CPU
// fallback.
#pragma once

#include <spg.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <new>
#include <optional>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

namespace spira {

// ---------------------------------------------------------------- tags/config
namespace layout::tags {
struct aos_tag {};
struct soa_tag {};
}  // namespace layout::tags

namespace layout {
template <class T>
concept ValidLayoutTag = std::is_same_v<T, tags::aos_tag> || std::is_same_v<T, tags::soa_tag>;

template <class I, class V>
struct elementPair {  // element_pair.hpp:8-18
    I column{};
    V value{};
};
}  // namespace layout

namespace config {
enum class matrix_mode : uint8_t { open, locked };                                   // config.hpp:14-17
enum class lock_policy : uint8_t { no_compact, compact_preserve, compact_move };     // config.hpp:23-27
enum class insert_policy : uint8_t { direct, staged };                               // config.hpp:33-40
}  // namespace config

namespace buffer::tags {
// Spira's row-buffer choices; on the GPU engine every policy stages inserts
// the same way, so the tags only keep user signatures compiling.
template <class LayoutTag = layout::tags::aos_tag>
struct array_buffer {};
struct hash_map_buffer {};
}  // namespace buffer::tags

namespace gpu {

// Maps a C ABI status to Spira's exception types.
inline void check(int status) {
    if (status == SPG_OK) return;
    const std::string msg = spg_last_error();
    switch (status) {
        case SPG_ERR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
        case SPG_ERR_LOGIC: throw std::logic_error(msg);
        case SPG_ERR_OUT_OF_RANGE: throw std::out_of_range(msg);
        case SPG_ERR_NO_MEMORY: throw std::bad_alloc();
        case SPG_ERR_DOMAIN: throw std::domain_error(msg);
        default: throw std::runtime_error(std::string(spg_strerror(status)) + ": " + msg);
    }
}

// One engine context per host thread (contexts are not thread-safe).
inline spg_ctx *context() {
    struct Holder {
        spg_ctx *c = nullptr;
        ~Holder() {
            if (c) spg_ctx_destroy(c);
        }
    };
    thread_local Holder h;
    if (!h.c) check(spg_ctx_create(0, &h.c));
    return h.c;
}

// Owning handle of a device CSR.
class csr_handle {
public:
    csr_handle() = default;
    csr_handle(std::size_t r, std::size_t c) { check(spg_csr_create(context(), r, c, &h_)); }
    csr_handle(const csr_handle &o) {
        if (o.h_) {
            spg_csr_info i;
            check(spg_csr_info_get(o.h_, &i));
            check(spg_csr_create(context(), i.n_rows, i.n_cols, &h_));
            check(spg_csr_copy(context(), o.h_, h_));
        }
    }
    csr_handle(csr_handle &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    csr_handle &operator=(csr_handle o) noexcept {
        std::swap(h_, o.h_);
        return *this;
    }
    ~csr_handle() {
        if (h_) spg_csr_destroy(h_);
    }
    spg_csr *get() const { return h_; }
    spg_csr_info info() const {
        spg_csr_info i{};
        check(spg_csr_info_get(h_, &i));
        return i;
    }

private:
    spg_csr *h_ = nullptr;
};

}  // namespace gpu

// ---------------------------------------------------------------- csr_storage
// Host view of the device CSR (csr_storage_soa.hpp:17-77 / csr_storage_aos.hpp:
// 18-67): returned by matrix::csr() as a snapshot, accepted by load_csr.
template <class LayoutTag, class I, class V>
struct csr_storage;

template <class I, class V>
struct csr_storage<layout::tags::soa_tag, I, V> {
    std::size_t n_rows{0}, nnz{0}, capacity{0};
    std::unique_ptr<std::size_t[]> offsets;
    std::unique_ptr<I[]> cols;
    std::unique_ptr<V[]> vals;
    csr_storage() = default;
    csr_storage(std::size_t r, std::size_t n) : csr_storage(r, n, n) {}
    csr_storage(std::size_t r, std::size_t n, std::size_t cap)
        : n_rows(r), nnz(n), capacity(cap), offsets(new std::size_t[r + 1]()), cols(new I[cap ? cap : 1]),
          vals(new V[cap ? cap : 1]) {}
    [[nodiscard]] bool is_built() const noexcept { return offsets != nullptr; }
};

template <class I, class V>
struct csr_storage<layout::tags::aos_tag, I, V> {
    std::size_t n_rows{0}, nnz{0}, capacity{0};
    std::unique_ptr<std::size_t[]> offsets;
    std::unique_ptr<layout::elementPair<I, V>[]> pairs;
    csr_storage() = default;
    csr_storage(std::size_t r, std::size_t n) : csr_storage(r, n, n) {}
    csr_storage(std::size_t r, std::size_t n, std::size_t cap)
        : n_rows(r), nnz(n), capacity(cap), offsets(new std::size_t[r + 1]()),
          pairs(new layout::elementPair<I, V>[cap ? cap : 1]) {}
    [[nodiscard]] bool is_built() const noexcept { return offsets != nullptr; }
};

// ---------------------------------------------------------------- matrix
template <class LayoutTag, class I = uint32_t, class V = double,
          class BufferTag = buffer::tags::array_buffer<layout::tags::aos_tag>, std::size_t BufferN = 64,
          config::lock_policy LP = config::lock_policy::compact_preserve>
    requires layout::ValidLayoutTag<LayoutTag>
class matrix {
    static_assert(std::is_same_v<I, uint32_t> && std::is_same_v<V, double>,
                  "the GB300 engine serves I = uint32_t, V = double");

public:
    using index_type = I;
    using value_type = V;
    using size_type = std::size_t;
    using shape_type = std::pair<size_type, size_type>;
    using storage = csr_storage<LayoutTag, I, V>;

    explicit matrix(size_type row_limit, size_type column_limit)
        : rows_(row_limit), cols_(column_limit), dev_(row_limit, column_limit) {}
    matrix(size_type row_limit, size_type column_limit, size_type /*reserve_per_row*/)
        : matrix(row_limit, column_limit) {}

    matrix(const matrix &o) = default;
    matrix(matrix &&) noexcept = default;
    matrix &operator=(const matrix &) = default;
    matrix &operator=(matrix &&) noexcept = default;

    // shape / mode
    [[nodiscard]] shape_type shape() const noexcept { return {rows_, cols_}; }
    [[nodiscard]] size_type n_rows() const noexcept { return rows_; }
    [[nodiscard]] size_type n_cols() const noexcept { return cols_; }
    [[nodiscard]] config::matrix_mode mode() const noexcept { return mode_; }
    [[nodiscard]] bool is_locked() const noexcept { return mode_ == config::matrix_mode::locked; }
    [[nodiscard]] bool is_open() const noexcept { return mode_ == config::matrix_mode::open; }

    // matrix.hpp:277-342: merge this epoch's staged inserts on the device.
    void lock() {
        if (is_locked()) return;
        gpu::check(spg_lock(gpu::context(), dev_.get(), st_rows_.data(), st_cols_.data(), st_vals_.data(),
                            st_rows_.size()));
        clear_staging();
        host_.reset();
        mode_ = config::matrix_mode::locked;
    }

    // matrix.hpp:348-357: committed CSR is kept as the next merge's base.
    void open() { mode_ = config::matrix_mode::open; }

    // matrix.hpp:453-462
    void insert(index_type r, index_type c, const value_type &v) {
        if (!is_open()) throw std::logic_error("matrix::insert() requires open mode");
        validate_row(r);
        validate_col(c);
        st_rows_.push_back(r);
        st_cols_.push_back(c);
        st_vals_.push_back(v);
    }

    void clear() {
        if (!is_open()) throw std::logic_error("matrix::clear() requires open mode");
        clear_staging();
    }

    // Open mode: upper bound (committed + staged, duplicates counted);
    // locked: exact (matrix.hpp:371-396).
    [[nodiscard]] size_type nnz() const { return dev_.info().nnz + (is_open() ? st_rows_.size() : 0); }
    [[nodiscard]] bool empty() const { return nnz() == 0; }
    [[nodiscard]] size_type row_nnz(index_type r) const {
        validate_row(r);
        uint64_t b = 0, e = 0;
        gpu::check(spg_csr_row_range(gpu::context(), dev_.get(), r, &b, &e));
        size_type n = e - b;
        if (is_open())
            for (auto rr : st_rows_) n += (rr == r);
        return n;
    }

    // row.hpp:178-206: open mode reads the staged buffer first (last write).
    [[nodiscard]] bool contains(index_type r, index_type c) const {
        validate_row(r);
        validate_col(c);
        if (is_open() && staged_index(r, c) >= 0) return true;
        double v;
        int f = 0;
        gpu::check(spg_csr_get(gpu::context(), dev_.get(), r, c, &v, &f));
        return f != 0;
    }

    [[nodiscard]] value_type get(index_type r, index_type c) const {
        validate_row(r);
        validate_col(c);
        if (is_open()) {
            const long k = staged_index(r, c);
            if (k >= 0) return st_vals_[static_cast<size_type>(k)];
        }
        double v = 0.0;
        int f = 0;
        gpu::check(spg_csr_get(gpu::context(), dev_.get(), r, c, &v, &f));
        return f ? v : 0.0;
    }

    // Host snapshot of the committed CSR (matrix.hpp:88-91), nullptr before
    // the first lock. Valid until the next lock / load_csr.
    [[nodiscard]] const storage *csr() const {
        const auto i = dev_.info();
        if (!i.built) return nullptr;
        if (!host_) {
            auto s = std::make_shared<storage>(i.n_rows, i.nnz, i.capacity);
            s->capacity = i.capacity;
            std::vector<uint64_t> off(i.n_rows + 1);
            std::vector<uint32_t> cc(i.nnz);
            std::vector<double> vv(i.nnz);
            gpu::check(spg_csr_download(gpu::context(), dev_.get(), off.data(), cc.data(), vv.data()));
            for (size_type k = 0; k <= i.n_rows; ++k) s->offsets[k] = off[k];
            if constexpr (std::is_same_v<LayoutTag, layout::tags::soa_tag>) {
                std::copy(cc.begin(), cc.end(), s->cols.get());
                std::copy(vv.begin(), vv.end(), s->vals.get());
            } else {
                for (size_type k = 0; k < i.nnz; ++k) s->pairs[k] = {cc[k], vv[k]};
            }
            host_ = s;
        }
        return host_.get();
    }

    // matrix.hpp:520-605: validated install; throws std::invalid_argument.
    void load_csr(storage &&s) {
        if (s.n_rows != rows_)
            throw std::invalid_argument("spira::matrix::load_csr: CSR row count does not match matrix dimensions");
        if (!s.offsets) throw std::invalid_argument("spira::matrix::load_csr: CSR offsets array is null");
        std::vector<uint64_t> off(s.offsets.get(), s.offsets.get() + s.n_rows + 1);
        if constexpr (std::is_same_v<LayoutTag, layout::tags::soa_tag>) {
            gpu::check(spg_csr_load(gpu::context(), dev_.get(), off.data(), s.cols.get(), s.vals.get(), s.nnz));
        } else {
            std::vector<uint32_t> cc(s.nnz);
            std::vector<double> vv(s.nnz);
            for (size_type k = 0; k < s.nnz; ++k) {
                cc[k] = s.pairs[k].column;
                vv[k] = s.pairs[k].value;
            }
            gpu::check(spg_csr_load(gpu::context(), dev_.get(), off.data(), cc.data(), vv.data(), s.nnz));
        }
        clear_staging();
        host_.reset();
        mode_ = config::matrix_mode::locked;
    }

    void swap(matrix &o) noexcept {
        using std::swap;
        swap(rows_, o.rows_);
        swap(cols_, o.cols_);
        swap(mode_, o.mode_);
        swap(dev_, o.dev_);
        swap(st_rows_, o.st_rows_);
        swap(st_cols_, o.st_cols_);
        swap(st_vals_, o.st_vals_);
        swap(host_, o.host_);
    }

    // matrix.hpp:438-443 via row.hpp:208-231. Locked: the row's committed
    // values summed left to right from 0 (on the device). Open: the staged
    // entries of the row (last write per column, in order of each column's
    // first insert: the iteration order of the row buffer's column index),
    // then the committed entries no staged entry shadows, in CSR order.
    [[nodiscard]] value_type accumulate(index_type r) const {
        validate_row(r);
        const auto i = dev_.info();
        if (is_locked() || st_rows_.empty()) {
            if (!i.built) return 0.0;
            double v = 0.0;
            gpu::check(spg_csr_row_sums_host(gpu::context(), dev_.get(), r, 1, &v));
            return v;
        }
        std::vector<uint32_t> order;  // columns by first staged insert
        std::vector<double> last;
        for (size_type k = 0; k < st_rows_.size(); ++k) {
            if (st_rows_[k] != r) continue;
            const auto it = std::find(order.begin(), order.end(), st_cols_[k]);
            if (it == order.end()) {
                order.push_back(st_cols_[k]);
                last.push_back(st_vals_[k]);
            } else {
                last[static_cast<size_type>(it - order.begin())] = st_vals_[k];
            }
        }
        double acc = 0.0;
        for (double v : last) acc += v;
        if (const auto *s = csr()) {
            for (std::size_t k = s->offsets[r]; k < s->offsets[r + 1]; ++k) {
                I col;
                V val;
                if constexpr (std::is_same_v<LayoutTag, layout::tags::soa_tag>) {
                    col = s->cols[k];
                    val = s->vals[k];
                } else {
                    col = s->pairs[k].column;
                    val = s->pairs[k].value;
                }
                if (std::find(order.begin(), order.end(), col) == order.end()) acc += val;
            }
        }
        return acc;
    }

    // Engine side of the in-place scalers (scalars.hpp:10-18, 37-49): every
    // committed value times / over s on the device, results that are +-0
    // removed. Staged inserts at committed positions are dropped (Spira
    // stages the scaled committed value after them, so it is the last write);
    // before the first lock the staged values themselves are scaled, as
    // Spira's row walks its buffer when no CSR slice is installed.
    void scale_in_place(value_type s, bool divide) {
        const auto i = dev_.info();
        if (!i.built) {
            for (auto &v : st_vals_) v = divide ? v / s : v * s;
            return;
        }
        if (!st_rows_.empty()) {
            const auto *snap = csr();
            size_type w = 0;
            for (size_type k = 0; k < st_rows_.size(); ++k) {
                const std::size_t b = snap->offsets[st_rows_[k]], e = snap->offsets[st_rows_[k] + 1];
                bool committed = false;
                for (std::size_t q = b; q < e && !committed; ++q) {
                    if constexpr (std::is_same_v<LayoutTag, layout::tags::soa_tag>) committed = snap->cols[q] == st_cols_[k];
                    else committed = snap->pairs[q].column == st_cols_[k];
                }
                if (committed) continue;
                st_rows_[w] = st_rows_[k];
                st_cols_[w] = st_cols_[k];
                st_vals_[w] = st_vals_[k];
                ++w;
            }
            st_rows_.resize(w);
            st_cols_.resize(w);
            st_vals_.resize(w);
        }
        gpu::check(spg_csr_scale(gpu::context(), dev_.get(), dev_.get(), s, divide ? 1 : 0));
        host_.reset();
    }

    // operators (matrix_operators.hpp:18-150)
    matrix operator+(const matrix &other) const;
    matrix operator-(const matrix &other) const;
    matrix &operator+=(const matrix &other);
    matrix &operator-=(const matrix &other);
    std::vector<value_type> operator*(const std::vector<value_type> &x) const;
    matrix operator*(const matrix &other) const;
    matrix &operator*=(const matrix &other) {
        *this = *this * other;
        return *this;
    }
    matrix operator*(value_type s) const;
    matrix &operator*=(value_type s);
    matrix operator/(value_type s) const;
    matrix &operator/=(value_type s);
    matrix operator~() const;

    // engine access
    [[nodiscard]] spg_csr *device_handle() const noexcept { return dev_.get(); }
    [[nodiscard]] bool csr_built() const { return dev_.info().built != 0; }
    [[nodiscard]] size_type staged_count() const noexcept { return st_rows_.size(); }
    // Adopts a device result (transpose / spgemm): locked, shape from the handle.
    static matrix adopt(gpu::csr_handle &&h) {
        const auto i = h.info();
        matrix m(i.n_rows, i.n_cols);
        m.dev_ = std::move(h);
        m.mode_ = config::matrix_mode::locked;
        return m;
    }

private:
    void validate_row(index_type r) const {
        if (static_cast<size_type>(r) >= rows_) throw std::out_of_range("spira::matrix: row_index out of range");
    }
    void validate_col(index_type c) const {
        if (static_cast<size_type>(c) >= cols_) throw std::out_of_range("spira::matrix: col_index out of range");
    }
    long staged_index(index_type r, index_type c) const {
        for (size_type k = st_rows_.size(); k-- > 0;)
            if (st_rows_[k] == r && st_cols_[k] == c) return static_cast<long>(k);
        return -1;
    }
    void clear_staging() {
        st_rows_.clear();
        st_cols_.clear();
        st_vals_.clear();
    }

    size_type rows_ = 0, cols_ = 0;
    config::matrix_mode mode_ = config::matrix_mode::open;
    gpu::csr_handle dev_;
    std::vector<uint32_t> st_rows_, st_cols_;
    std::vector<double> st_vals_;
    mutable std::shared_ptr<storage> host_;
};

// ---------------------------------------------------------------- serial algorithms
namespace serial::algorithms {

// serial/spmv.hpp:141-186 (checks in the same order, same messages).
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void spmv(const spira::matrix<L, I, V, BT, BN, LP> &mat, const std::vector<V> &x, std::vector<V> &y,
                 int variant = SPG_SPMV_AUTO) {
    if (x.size() != mat.n_cols())
        throw std::invalid_argument(
            "The size of the input vector x does not match the number of columns of the matrix");
    if (y.size() != mat.n_rows())
        throw std::invalid_argument(
            "The size of the output vector y does not match the number of rows of the matrix");
    if (!mat.is_locked()) throw std::logic_error("spmv: matrix must be locked");
    gpu::check(spg_spmv_host(gpu::context(), mat.device_handle(), x.data(), x.size(), y.data(), y.size(), variant));
}

// serial/spgemm.hpp:12-53
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline spira::matrix<L, I, V, BT, BN, LP> spgemm(const spira::matrix<L, I, V, BT, BN, LP> &A,
                                                 const spira::matrix<L, I, V, BT, BN, LP> &B) {
    if (A.n_cols() != B.n_rows()) throw std::invalid_argument("A.cols must equal B.rows");
    if (!A.is_locked()) throw std::logic_error("spgemm: A must be locked");
    if (!B.is_locked()) throw std::logic_error("spgemm: B must be locked");
    gpu::csr_handle out(A.n_rows(), B.n_cols());
    gpu::check(spg_spgemm(gpu::context(), A.device_handle(), B.device_handle(), out.get()));
    return spira::matrix<L, I, V, BT, BN, LP>::adopt(std::move(out));
}

// serial/transpose.hpp:35-156
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline spira::matrix<L, I, V, BT, BN, LP> transpose(const spira::matrix<L, I, V, BT, BN, LP> &mat) {
    if (!mat.is_locked()) throw std::logic_error("transpose: matrix must be locked");
    gpu::csr_handle out(mat.n_cols(), mat.n_rows());
    gpu::check(spg_transpose(gpu::context(), mat.device_handle(), out.get()));
    return spira::matrix<L, I, V, BT, BN, LP>::adopt(std::move(out));
}

// serial/transpose.hpp:159-172
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void transpose_itself(spira::matrix<L, I, V, BT, BN, LP> &mat) {
    if (!mat.is_open()) throw std::logic_error("transpose_itself: matrix must be open");
    auto [r, c] = mat.shape();
    if (r != c) throw std::logic_error("in-place transpose requires square matrix");
    mat.lock();
    auto out = transpose(mat);
    mat.swap(out);
    mat.open();
}

// serial/matrix_addition.hpp:86-110 (checks in the same order).
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline spira::matrix<L, I, V, BT, BN, LP> MatrixAddition(const spira::matrix<L, I, V, BT, BN, LP> &A,
                                                         const spira::matrix<L, I, V, BT, BN, LP> &B) {
    if (A.shape() != B.shape()) throw std::invalid_argument("Matrices aren't the same size");
    if (!A.is_locked()) throw std::logic_error("MatrixAddition: A must be locked");
    if (!B.is_locked()) throw std::logic_error("MatrixAddition: B must be locked");
    gpu::csr_handle out(A.n_rows(), A.n_cols());  // (a locked matrix always holds a device CSR)
    gpu::check(spg_csr_add(gpu::context(), A.device_handle(), B.device_handle(), out.get()));
    return spira::matrix<L, I, V, BT, BN, LP>::adopt(std::move(out));
}

// serial/scalars.hpp:9-18 (in place: the matrix must be open).
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void multiplication_scaler(spira::matrix<L, I, V, BT, BN, LP> &mat, V scaler) {
    if (!mat.is_open()) throw std::logic_error("multiplication_scaler: matrix must be open");
    mat.scale_in_place(scaler, false);
}

// serial/scalars.hpp:22-35 (copy path: mat locked, out replaced).
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void multiplication_scaler(const spira::matrix<L, I, V, BT, BN, LP> &mat, spira::matrix<L, I, V, BT, BN, LP> &out,
                                  V scaler) {
    if (!mat.is_locked()) throw std::logic_error("multiplication_scaler: input matrix must be locked");
    gpu::csr_handle h(mat.n_rows(), mat.n_cols());
    gpu::check(spg_csr_scale(gpu::context(), mat.device_handle(), h.get(), scaler, 0));
    out = spira::matrix<L, I, V, BT, BN, LP>::adopt(std::move(h));
}

// serial/scalars.hpp:37-49: the zero check fires before the mode check.
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void division_scaler(spira::matrix<L, I, V, BT, BN, LP> &mat, V scaler) {
    if (std::fabs(scaler) <= 0.0) throw std::domain_error("Divison by zero");
    if (!mat.is_open()) throw std::logic_error("division_scaler: matrix must be open");
    mat.scale_in_place(scaler, true);
}

// serial/scalars.hpp:51-67
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline void division_scaler(const spira::matrix<L, I, V, BT, BN, LP> &mat, spira::matrix<L, I, V, BT, BN, LP> &out,
                            V scaler) {
    if (std::fabs(scaler) <= 0.0) throw std::domain_error("Divison by zero");
    if (!mat.is_locked()) throw std::logic_error("division_scaler: input matrix must be locked");
    gpu::csr_handle h(mat.n_rows(), mat.n_cols());
    gpu::check(spg_csr_scale(gpu::context(), mat.device_handle(), h.get(), scaler, 1));
    out = spira::matrix<L, I, V, BT, BN, LP>::adopt(std::move(h));
}

// serial/accumulate.hpp:12-32
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline V accumulate(const spira::matrix<L, I, V, BT, BN, LP> &mat, std::size_t i) {
    if (i >= mat.shape().first) throw std::out_of_range("Row does not exist in matrix");
    return mat.accumulate(static_cast<I>(i));
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
inline std::vector<V> accumulate(const spira::matrix<L, I, V, BT, BN, LP> &mat) {
    std::vector<V> acc(mat.n_rows(), 0.0);
    if (mat.n_rows() == 0) return acc;
    if (mat.csr_built() && (mat.is_locked() || mat.staged_count() == 0)) {  // every row at once, on the device
        gpu::check(spg_csr_row_sums_host(gpu::context(), mat.device_handle(), 0, mat.n_rows(), acc.data()));
        return acc;
    }
    for (std::size_t r = 0; r < mat.n_rows(); ++r) acc[r] = mat.accumulate(static_cast<I>(r));
    return acc;
}

}  // namespace serial::algorithms

// matrix_operators.hpp:18-62: A - B is A + (B * -1).
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator+(const matrix &other) const {
    return serial::algorithms::MatrixAddition(*this, other);
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator-(const matrix &other) const {
    if (this->shape() != other.shape()) throw std::invalid_argument("operator-: matrix shapes must match");
    matrix out(other.n_rows(), other.n_cols());
    serial::algorithms::multiplication_scaler(other, out, V{-1});
    return serial::algorithms::MatrixAddition(*this, out);
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> &matrix<L, I, V, BT, BN, LP>::operator+=(const matrix &other) {
    *this = serial::algorithms::MatrixAddition(*this, other);
    return *this;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> &matrix<L, I, V, BT, BN, LP>::operator-=(const matrix &other) {
    if (this->shape() != other.shape()) throw std::invalid_argument("operator-=: matrix shapes must match");
    matrix out(other.n_rows(), other.n_cols());
    serial::algorithms::multiplication_scaler(other, out, V{-1});
    *this = serial::algorithms::MatrixAddition(*this, out);
    return *this;
}

// matrix_operators.hpp:104-140
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator*(V s) const {
    matrix out(n_rows(), n_cols());
    serial::algorithms::multiplication_scaler(*this, out, s);
    return out;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> &matrix<L, I, V, BT, BN, LP>::operator*=(V s) {
    serial::algorithms::multiplication_scaler(*this, s);
    return *this;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator/(V s) const {
    matrix out(n_rows(), n_cols());
    serial::algorithms::division_scaler(*this, out, s);
    return out;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> &matrix<L, I, V, BT, BN, LP>::operator/=(V s) {
    serial::algorithms::division_scaler(*this, s);
    return *this;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline std::vector<V> matrix<L, I, V, BT, BN, LP>::operator*(const std::vector<V> &x) const {
    std::vector<V> y(n_rows());
    serial::algorithms::spmv(*this, x, y);
    return y;
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator*(const matrix &other) const {
    return serial::algorithms::spgemm(*this, other);
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP>
    requires layout::ValidLayoutTag<L>
inline matrix<L, I, V, BT, BN, LP> matrix<L, I, V, BT, BN, LP>::operator~() const {
    return serial::algorithms::transpose(*this);
}

// ---------------------------------------------------------------- parallel
namespace parallel {

// partition.hpp:78-126: nnz-balanced boundaries by prefix sum + lower_bound.
inline std::vector<std::size_t> compute_partition_boundaries(const std::vector<std::size_t> &row_nnz,
                                                             std::size_t n_threads) {
    const std::size_t n_rows = row_nnz.size();
    std::vector<std::size_t> b(n_threads + 1, n_rows);
    b[0] = 0;
    if (n_threads <= 1 || n_rows == 0) return b;
    std::vector<std::size_t> prefix(n_rows + 1, 0);
    for (std::size_t i = 0; i < n_rows; ++i) prefix[i + 1] = prefix[i] + row_nnz[i];
    const std::size_t total = prefix[n_rows];
    if (total == 0) {
        for (std::size_t t = 1; t < n_threads; ++t) b[t] = t * n_rows / n_threads;
        return b;
    }
    for (std::size_t t = 1; t < n_threads; ++t) {
        const std::size_t target = std::max<std::size_t>(1, t * total / n_threads);
        auto it = std::lower_bound(prefix.cbegin() + static_cast<std::ptrdiff_t>(b[t - 1]), prefix.cend(), target);
        b[t] = std::min(static_cast<std::size_t>(it - prefix.cbegin()), n_rows);
    }
    return b;
}

// A partition's rows as parallel_fill hands them out: rows[local].insert().
template <class I, class V>
class row_stage {
public:
    row_stage(std::size_t global_row, std::size_t n_cols, std::vector<uint32_t> *r, std::vector<uint32_t> *c,
              std::vector<double> *v)
        : g_(global_row), n_cols_(n_cols), r_(r), c_(c), v_(v) {}
    void insert(I col, V val) {  // row.hpp:162-169
        if (static_cast<std::size_t>(col) >= n_cols_) throw std::out_of_range("Column index out of range");
        r_->push_back(static_cast<uint32_t>(g_));
        c_->push_back(col);
        v_->push_back(val);
    }

private:
    std::size_t g_, n_cols_;
    std::vector<uint32_t> *r_, *c_;
    std::vector<double> *v_;
};

template <class L, class I, class V>
struct partition {  // partition.hpp:32-58 (rows are staging proxies; csr is a host snapshot)
    std::size_t row_start{0}, row_end{0};
    std::vector<row_stage<I, V>> rows{};
    csr_storage<L, I, V> csr{};
    [[nodiscard]] std::size_t size() const noexcept { return row_end - row_start; }
    [[nodiscard]] std::size_t local_row(std::size_t g) const noexcept { return g - row_start; }
};

template <class LayoutTag, class I = uint32_t, class V = double,
          class BufferTag = buffer::tags::array_buffer<layout::tags::aos_tag>, std::size_t BufferN = 64,
          config::lock_policy LP = config::lock_policy::compact_preserve,
          config::insert_policy IP = config::insert_policy::direct, std::size_t StagingN = 256>
    requires layout::ValidLayoutTag<LayoutTag>
class parallel_matrix {
    using base_matrix = spira::matrix<LayoutTag, I, V, BufferTag, BufferN, LP>;

public:
    using base_type = base_matrix;
    using index_type = I;
    using value_type = V;
    using size_type = std::size_t;
    using partition_type = partition<LayoutTag, I, V>;

    parallel_matrix(size_type n_rows, size_type n_cols, size_type n_threads)
        : m_(n_rows, n_cols), n_threads_(n_threads) {
        if (n_threads < 1) throw std::invalid_argument("parallel_matrix requires at least one thread");
        bounds_.resize(n_threads + 1);
        for (size_type t = 0; t <= n_threads; ++t) bounds_[t] = t * n_rows / n_threads;  // parallel_matrix.hpp:300-301
    }
    parallel_matrix(size_type n_rows, size_type n_cols, size_type n_threads, size_type)
        : parallel_matrix(n_rows, n_cols, n_threads) {}
    parallel_matrix(const parallel_matrix &) = delete;
    parallel_matrix &operator=(const parallel_matrix &) = delete;
    parallel_matrix(parallel_matrix &&) = default;
    parallel_matrix &operator=(parallel_matrix &&) = default;

    [[nodiscard]] size_type n_rows() const noexcept { return m_.n_rows(); }
    [[nodiscard]] size_type n_cols() const noexcept { return m_.n_cols(); }
    [[nodiscard]] size_type n_threads() const noexcept { return n_threads_; }
    [[nodiscard]] std::pair<size_type, size_type> shape() const noexcept { return m_.shape(); }
    [[nodiscard]] config::matrix_mode mode() const noexcept { return m_.mode(); }
    [[nodiscard]] bool is_locked() const noexcept { return m_.is_locked(); }
    [[nodiscard]] bool is_open() const noexcept { return m_.is_open(); }

    void insert(size_type r, I c, V v) {
        if (!is_open()) throw std::logic_error("parallel_matrix::insert() requires open mode");
        if (r >= n_rows()) throw std::out_of_range("parallel_matrix: row index out of range");
        if (static_cast<size_type>(c) >= n_cols()) throw std::out_of_range("parallel_matrix: col index out of range");
        m_.insert(static_cast<I>(r), c, v);
    }

    // parallel_matrix.hpp:179-189: f(rows, row_start, row_end, thread_id) on
    // one host thread per partition; every partition stages into its own
    // arrays, appended in partition order at the end.
    template <class Func>
    void parallel_fill(Func &&f) {
        if (!is_open()) throw std::logic_error("parallel_fill: matrix must be open");
        std::vector<std::vector<uint32_t>> R(n_threads_), C(n_threads_);
        std::vector<std::vector<double>> Vv(n_threads_);
        std::vector<std::thread> th;
        std::vector<std::exception_ptr> err(n_threads_);
        for (size_type t = 0; t < n_threads_; ++t)
            th.emplace_back([&, t] {
                try {
                    std::vector<row_stage<I, V>> rows;
                    for (size_type g = bounds_[t]; g < bounds_[t + 1]; ++g)
                        rows.emplace_back(g, n_cols(), &R[t], &C[t], &Vv[t]);
                    f(rows, bounds_[t], bounds_[t + 1], t);
                } catch (...) {
                    err[t] = std::current_exception();
                }
            });
        for (auto &x : th) x.join();
        for (auto &e : err)
            if (e) std::rethrow_exception(e);
        for (size_type t = 0; t < n_threads_; ++t)
            for (size_type k = 0; k < R[t].size(); ++k) m_.insert(R[t][k], C[t][k], Vv[t][k]);
    }

    void lock() { m_.lock(); }
    void open() { m_.open(); }
    void clear() { m_.clear(); }

    // parallel_matrix.hpp:434-497: nnz-balanced partition boundaries
    // (partition.hpp:78-126) computed on the device from the CSR offsets. The
    // device CSR is one array, so only the bookkeeping moves.
    void rebalance() {
        if (!is_locked()) throw std::logic_error("rebalance: matrix must be locked");
        std::vector<uint64_t> b(n_threads_ + 1);
        gpu::check(spg_csr_partition(gpu::context(), m_.device_handle(), n_threads_, b.data()));
        for (size_type t = 0; t <= n_threads_; ++t) bounds_[t] = static_cast<size_type>(b[t]);
    }

    // parallel_matrix.hpp:568-580
    [[nodiscard]] V accumulate(size_type r) const {
        if (r >= n_rows()) throw std::out_of_range("parallel_matrix: row index out of range");
        return m_.accumulate(static_cast<I>(r));
    }

    [[nodiscard]] size_type nnz() const { return m_.nnz(); }
    [[nodiscard]] bool empty() const { return m_.empty(); }
    [[nodiscard]] size_type row_nnz(size_type r) const {
        if (r >= n_rows()) throw std::out_of_range("parallel_matrix: row index out of range");
        return m_.row_nnz(static_cast<I>(r));
    }
    [[nodiscard]] bool contains(size_type r, I c) const {
        if (r >= n_rows()) throw std::out_of_range("parallel_matrix: row index out of range");
        if (static_cast<size_type>(c) >= n_cols()) throw std::out_of_range("parallel_matrix: col index out of range");
        return m_.contains(static_cast<I>(r), c);
    }
    [[nodiscard]] V get(size_type r, I c) const {
        if (r >= n_rows()) throw std::out_of_range("parallel_matrix: row index out of range");
        if (static_cast<size_type>(c) >= n_cols()) throw std::out_of_range("parallel_matrix: col index out of range");
        return m_.get(static_cast<I>(r), c);
    }

    // Host snapshot of partition t (row range + its CSR slice).
    [[nodiscard]] partition_type partition_at(size_type t) const {
        if (t >= n_threads_) throw std::out_of_range("parallel_matrix::partition_at: thread index out of range");
        partition_type p;
        p.row_start = bounds_[t];
        p.row_end = bounds_[t + 1];
        if (const auto *s = m_.csr()) {
            const size_type b = s->offsets[p.row_start], e = s->offsets[p.row_end];
            p.csr = csr_storage<LayoutTag, I, V>(p.size(), e - b);
            for (size_type i = 0; i <= p.size(); ++i) p.csr.offsets[i] = s->offsets[p.row_start + i] - b;
            if constexpr (std::is_same_v<LayoutTag, layout::tags::soa_tag>) {
                std::copy(s->cols.get() + b, s->cols.get() + e, p.csr.cols.get());
                std::copy(s->vals.get() + b, s->vals.get() + e, p.csr.vals.get());
            } else {
                std::copy(s->pairs.get() + b, s->pairs.get() + e, p.csr.pairs.get());
            }
        }
        return p;
    }

    template <class Func>
    void execute(Func &&f) {
        for (size_type t = 0; t < n_threads_; ++t) {
            auto p = partition_at(t);
            f(p, t);
        }
    }

    [[nodiscard]] const base_matrix &engine_matrix() const noexcept { return m_; }
    [[nodiscard]] base_matrix &engine_matrix() noexcept { return m_; }
    static parallel_matrix adopt(base_matrix &&m, size_type n_threads) {
        parallel_matrix p(m.n_rows(), m.n_cols(), n_threads);
        p.m_ = std::move(m);
        return p;
    }

private:
    base_matrix m_;
    size_type n_threads_;
    std::vector<size_type> bounds_;
};

namespace algorithms {

// parallel/algorithms/spmv.hpp:125-161
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void spmv(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat, const std::vector<V> &x, std::vector<V> &y) {
    if (x.size() != mat.n_cols()) throw std::invalid_argument("spmv: x size does not match matrix column count");
    if (y.size() != mat.n_rows()) throw std::invalid_argument("spmv: y size does not match matrix row count");
    if (!mat.is_locked()) throw std::logic_error("spmv: matrix must be locked");
    gpu::check(spg_spmv_host(gpu::context(), mat.engine_matrix().device_handle(), x.data(), x.size(), y.data(),
                             y.size(), SPG_SPMV_AUTO));
}

// parallel/algorithms/spgemm.hpp:27-69
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline parallel_matrix<L, I, V, BT, BN, LP, IP, SN> spgemm(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &A,
                                                           parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &B) {
    if (A.n_cols() != B.n_rows()) throw std::invalid_argument("spgemm: A.n_cols() must equal B.n_rows()");
    if (!A.is_locked()) throw std::logic_error("spgemm: A must be locked");
    if (!B.is_locked()) throw std::logic_error("spgemm: B must be locked");
    auto m = serial::algorithms::spgemm(A.engine_matrix(), B.engine_matrix());
    return parallel_matrix<L, I, V, BT, BN, LP, IP, SN>::adopt(std::move(m), A.n_threads());
}

// parallel/algorithms/transpose.hpp:36-70
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline parallel_matrix<L, I, V, BT, BN, LP, IP, SN> transpose(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat) {
    if (!mat.is_locked()) throw std::logic_error("transpose: matrix must be locked");
    auto m = serial::algorithms::transpose(mat.engine_matrix());
    return parallel_matrix<L, I, V, BT, BN, LP, IP, SN>::adopt(std::move(m), mat.n_threads());
}

// parallel/algorithms/matrix_addition.hpp:24-99
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline parallel_matrix<L, I, V, BT, BN, LP, IP, SN> MatrixAddition(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &A,
                                                                   parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &B) {
    if (A.shape() != B.shape()) throw std::invalid_argument("MatrixAddition: matrices must have the same shape");
    if (A.n_threads() != B.n_threads())
        throw std::invalid_argument("MatrixAddition: matrices must have the same thread count");
    if (!A.is_locked()) throw std::logic_error("MatrixAddition: A must be locked");
    if (!B.is_locked()) throw std::logic_error("MatrixAddition: B must be locked");
    auto m = serial::algorithms::MatrixAddition(A.engine_matrix(), B.engine_matrix());
    return parallel_matrix<L, I, V, BT, BN, LP, IP, SN>::adopt(std::move(m), A.n_threads());
}

// parallel/algorithms/scalars.hpp:16-31, 69-84 (in place; open matrix)
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void multiplication_scaler(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat, V scaler) {
    if (!mat.is_open()) throw std::logic_error("multiplication_scaler: matrix must be open");
    mat.engine_matrix().scale_in_place(scaler, false);
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void division_scaler(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat, V scaler) {
    if (std::fabs(scaler) <= 0.0) throw std::domain_error("division by zero");
    if (!mat.is_open()) throw std::logic_error("division_scaler: matrix must be open");
    mat.engine_matrix().scale_in_place(scaler, true);
}

// parallel/algorithms/scalars.hpp:37-62, 91-116 (copy: mat locked, out open,
// same shape and thread count; out ends locked)
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void scale_into(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat,
                       parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &out, V scaler, bool divide, const char *who) {
    if (!mat.is_locked()) throw std::logic_error(std::string(who) + ": input matrix must be locked");
    if (!out.is_open()) throw std::logic_error(std::string(who) + ": output matrix must be open");
    if (mat.shape() != out.shape()) throw std::invalid_argument(std::string(who) + ": shape mismatch");
    if (mat.n_threads() != out.n_threads()) throw std::invalid_argument(std::string(who) + ": thread count mismatch");
    typename parallel_matrix<L, I, V, BT, BN, LP, IP, SN>::base_type r(mat.n_rows(), mat.n_cols());
    if (divide) serial::algorithms::division_scaler(mat.engine_matrix(), r, scaler);
    else serial::algorithms::multiplication_scaler(mat.engine_matrix(), r, scaler);
    out = parallel_matrix<L, I, V, BT, BN, LP, IP, SN>::adopt(std::move(r), out.n_threads());
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void multiplication_scaler(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat,
                                  parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &out, V scaler) {
    scale_into(mat, out, scaler, false, "multiplication_scaler");
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline void division_scaler(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat,
                            parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &out, V scaler) {
    if (std::fabs(scaler) <= 0.0) throw std::domain_error("division by zero");
    scale_into(mat, out, scaler, true, "division_scaler");
}

// parallel/algorithms/accumulate.hpp:16-53
template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline V accumulate(const parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat, std::size_t row) {
    if (row >= mat.n_rows()) throw std::out_of_range("accumulate: row index out of range");
    return mat.accumulate(row);
}

template <class L, class I, class V, class BT, std::size_t BN, config::lock_policy LP, config::insert_policy IP,
          std::size_t SN>
inline std::vector<V> accumulate(parallel_matrix<L, I, V, BT, BN, LP, IP, SN> &mat) {
    return serial::algorithms::accumulate(mat.engine_matrix());
}

}  // namespace algorithms
}  // namespace parallel
}  // namespace spira
