// test_facade.cpp — Spira's own test scenarios, unchanged in spelling, run
// against the GB300 facade (include/spira_gb300/spira.hpp). Each TEST names
// the Spira test it restates. A tiny runner stands in for GoogleTest (absent
// offline); exit status is the number of failed tests.
#include <spira_gb300/spira.hpp>

#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

namespace {

struct Case {
    const char *name;
    std::function<void()> fn;
};
std::vector<Case> &registry() {
    static std::vector<Case> r;
    return r;
}
struct Reg {
    Reg(const char *n, std::function<void()> f) { registry().push_back({n, std::move(f)}); }
};
int g_fail = 0;
bool g_case_failed = false;

#define TEST(a, b) \
    static void a##_##b(); \
    static Reg reg_##a##_##b(#a "." #b, a##_##b); \
    static void a##_##b()
#define EXPECT_TRUE(x) \
    do { if (!(x)) { std::printf("  %s:%d: EXPECT_TRUE(%s)\n", __FILE__, __LINE__, #x); g_case_failed = true; } } while (0)
#define EXPECT_FALSE(x) EXPECT_TRUE(!(x))
#define EXPECT_EQ(a, b) \
    do { if (!((a) == (b))) { std::printf("  %s:%d: EXPECT_EQ(%s, %s)\n", __FILE__, __LINE__, #a, #b); g_case_failed = true; } } while (0)
#define EXPECT_DOUBLE_EQ(a, b) \
    do { const double _a = (a), _b = (b); \
         if (!(_a == _b || std::fabs(_a - _b) <= 4 * 2.220446049250313e-16 * std::max(std::fabs(_a), std::fabs(_b)))) { \
             std::printf("  %s:%d: EXPECT_DOUBLE_EQ(%s, %s): %.17g vs %.17g\n", __FILE__, __LINE__, #a, #b, _a, _b); \
             g_case_failed = true; } } while (0)
#define EXPECT_NEAR(a, b, t) \
    do { if (!(std::fabs((a) - (b)) <= (t))) { std::printf("  %s:%d: EXPECT_NEAR(%s, %s)\n", __FILE__, __LINE__, #a, #b); g_case_failed = true; } } while (0)
#define EXPECT_THROW(stmt, ex) \
    do { bool _ok = false; try { stmt; } catch (const ex &) { _ok = true; } catch (...) {} \
         if (!_ok) { std::printf("  %s:%d: EXPECT_THROW(%s, %s)\n", __FILE__, __LINE__, #stmt, #ex); g_case_failed = true; } } while (0)

using SoA = spira::layout::tags::soa_tag;
using AoS = spira::layout::tags::aos_tag;
using MS = spira::matrix<SoA, uint32_t, double>;
using MA = spira::matrix<AoS, uint32_t, double>;

template <class M>
std::vector<double> dense_ref(const M &A, const std::vector<double> &x) {
    std::vector<double> y(A.n_rows(), 0.0);
    for (std::size_t r = 0; r < A.n_rows(); ++r)
        for (std::size_t c = 0; c < A.n_cols(); ++c) y[r] += A.get(r, c) * x[c];
    return y;
}

}  // namespace

// tests/serial/spmv_tests.cpp:141-187
TEST(SpmvAccuracyTest, RectangularOutOfOrderDouble) {
    MS A(3, 5);
    A.insert(0, 0, 1.0);
    A.insert(0, 3, 2.0);
    A.insert(1, 2, 3.0);
    A.insert(2, 4, 5.0);
    A.insert(2, 1, 4.0);
    A.lock();
    std::vector<double> x = {1, 2, 3, 4, 5}, y(3, 0.0);
    spira::serial::algorithms::spmv(A, x, y);
    EXPECT_DOUBLE_EQ(y[0], 9.0);
    EXPECT_DOUBLE_EQ(y[1], 9.0);
    EXPECT_DOUBLE_EQ(y[2], 33.0);
}

// tests/serial/spmv_tests.cpp:189-237
TEST(SpmvAccuracyTest, MatchesDenseReference_MixedPattern_AOS) {
    MA A(5, 6);
    A.insert(0, 1, 2.0);
    A.insert(0, 4, -1.0);
    A.insert(1, 0, 3.5);
    A.insert(2, 5, 7.0);
    A.insert(3, 2, 1.25);
    A.insert(3, 2, 4.0);  // last write wins
    A.insert(4, 3, -2.0);
    A.lock();
    std::vector<double> x = {1, 2, 3, 4, 5, 6}, y(5, 0.0);
    auto ref = dense_ref(A, x);
    spira::serial::algorithms::spmv(A, x, y);
    for (int i = 0; i < 5; ++i) EXPECT_DOUBLE_EQ(y[i], ref[i]);
    EXPECT_DOUBLE_EQ(A.get(3, 2), 4.0);
}

// tests/serial/spmv_tests.cpp:239-299
TEST(SpmvAccuracyTest, EmptyMatrixAndDimensionMismatch) {
    MS A(4, 5);
    A.lock();
    std::vector<double> x(5, 3.14), y(4, 123.0);
    spira::serial::algorithms::spmv(A, x, y);
    for (auto v : y) EXPECT_DOUBLE_EQ(v, 0.0);
    MS B(3, 4);
    std::vector<double> xb(3, 1.0), yy(3, 0.0);
    EXPECT_THROW(spira::serial::algorithms::spmv(B, xb, yy), std::invalid_argument);
    std::vector<double> x4(4, 1.0), yb(2, 0.0);
    EXPECT_THROW(spira::serial::algorithms::spmv(B, x4, yb), std::invalid_argument);
    EXPECT_THROW(spira::serial::algorithms::spmv(B, x4, yy), std::logic_error);  // not locked
}

// tests/flush_behaviour_tests.cpp:17-52
TEST(LockBehaviorTest, SingleLock_DedupLastWriteWins) {
    MS mat(1, 10);
    mat.insert(0, 1, 1.0);
    mat.insert(0, 2, 2.0);
    mat.insert(0, 3, 3.0);
    mat.insert(0, 4, 4.0);
    mat.insert(0, 1, 5.0);
    mat.lock();
    EXPECT_DOUBLE_EQ(mat.get(0, 1), 5.0);
    EXPECT_TRUE(mat.contains(0, 2));
    EXPECT_EQ(mat.row_nnz(0), 4u);
    EXPECT_EQ(mat.nnz(), 4u);
}

// tests/flush_behaviour_tests.cpp:96-176
TEST(LockBehaviorTest, IncrementalMergeAndOverwrite) {
    MA mat(1, 10);
    mat.insert(0, 3, 4.0);
    mat.insert(0, 5, 99.0);
    mat.lock();
    EXPECT_EQ(mat.row_nnz(0), 2u);
    mat.open();
    mat.insert(0, 9, 7.0);
    mat.insert(0, 5, 2.0);
    mat.lock();
    EXPECT_EQ(mat.row_nnz(0), 3u);
    EXPECT_DOUBLE_EQ(mat.get(0, 3), 4.0);
    EXPECT_DOUBLE_EQ(mat.get(0, 5), 2.0);
    EXPECT_DOUBLE_EQ(mat.get(0, 9), 7.0);
}

// tests/flush_behaviour_tests.cpp:178-276
TEST(LockBehaviorTest, ZeroFilteredAndZeroDeletes) {
    MS mat(2, 10);
    mat.insert(0, 1, 5.0);
    mat.insert(0, 2, 0.0);
    mat.insert(1, 3, 3.0);
    mat.lock();
    EXPECT_EQ(mat.row_nnz(0), 1u);
    EXPECT_FALSE(mat.contains(0, 2));
    mat.open();
    mat.insert(0, 1, 0.0);
    mat.insert(1, 3, -0.0);
    mat.lock();
    EXPECT_EQ(mat.nnz(), 0u);
    EXPECT_FALSE(mat.contains(0, 1));
    EXPECT_DOUBLE_EQ(mat.get(1, 3), 0.0);
}

// tests/flush_behaviour_tests.cpp:278-296
TEST(LockBehaviorTest, OpenModeGet_BufferFirst_ThenSlab) {
    MA mat(1, 10);
    mat.insert(0, 7, 1.0);
    mat.lock();
    mat.open();
    mat.insert(0, 7, 9.0);
    EXPECT_DOUBLE_EQ(mat.get(0, 7), 9.0);
    mat.lock();
    EXPECT_DOUBLE_EQ(mat.get(0, 7), 9.0);
}

// tests/matrix_tests.cpp (mode and bounds errors)
TEST(MatrixTest, ModeAndBoundsErrors) {
    MS mat(2, 3);
    EXPECT_THROW(mat.insert(2, 0, 1.0), std::out_of_range);
    EXPECT_THROW(mat.insert(0, 3, 1.0), std::out_of_range);
    mat.lock();
    EXPECT_THROW(mat.insert(0, 0, 1.0), std::logic_error);
    EXPECT_THROW((void)mat.get(5, 0), std::out_of_range);
}

// tests/compaction_tests.cpp:71-100 through csr()
TEST(BuildCSR, MultipleRowsMultipleEntries_OffsetsColsValsExact) {
    MA mat(3, 5);
    mat.insert(0, 0, 1.0);
    mat.insert(0, 3, 2.0);
    mat.insert(1, 1, 3.0);
    mat.insert(2, 2, 4.0);
    mat.lock();
    const auto *csr = mat.csr();
    EXPECT_TRUE(csr != nullptr);
    EXPECT_EQ(csr->nnz, 4u);
    EXPECT_EQ(csr->offsets[1], 2u);
    EXPECT_EQ(csr->offsets[3], 4u);
    EXPECT_EQ(csr->pairs[1].column, 3u);
    EXPECT_DOUBLE_EQ(csr->pairs[2].value, 3.0);
}

// matrix.hpp:520-605 load_csr validation
TEST(LoadCsr, ValidatesAndInstalls) {
    MS m(2, 3);
    spira::csr_storage<SoA, uint32_t, double> bad(2, 2);
    bad.offsets[0] = 0; bad.offsets[1] = 2; bad.offsets[2] = 2;
    bad.cols[0] = 2; bad.cols[1] = 1;  // not sorted
    bad.vals[0] = 1.0; bad.vals[1] = 2.0;
    EXPECT_THROW(m.load_csr(std::move(bad)), std::invalid_argument);
    spira::csr_storage<SoA, uint32_t, double> ok(2, 2);
    ok.offsets[0] = 0; ok.offsets[1] = 1; ok.offsets[2] = 2;
    ok.cols[0] = 2; ok.cols[1] = 0;
    ok.vals[0] = 1.5; ok.vals[1] = -2.0;
    m.load_csr(std::move(ok));
    EXPECT_TRUE(m.is_locked());
    EXPECT_DOUBLE_EQ(m.get(0, 2), 1.5);
    EXPECT_DOUBLE_EQ(m.get(1, 0), -2.0);
}

// tests/serial/spgemm_tests.cpp:130-151, 189-202
TEST(SpGEMM, SmallExampleAndAccumulation) {
    MS A(2, 3), B(3, 2);
    A.insert(0, 0, 1); A.insert(0, 2, 2); A.insert(1, 1, 3);
    B.insert(0, 1, 4); B.insert(1, 0, 5); B.insert(2, 1, 6);
    A.lock();
    B.lock();
    auto C = A * B;
    EXPECT_EQ(C.n_rows(), 2u);
    EXPECT_EQ(C.n_cols(), 2u);
    EXPECT_DOUBLE_EQ(C.get(0, 0), 0.0);
    EXPECT_DOUBLE_EQ(C.get(0, 1), 16.0);
    EXPECT_DOUBLE_EQ(C.get(1, 0), 15.0);
    EXPECT_FALSE(C.contains(1, 1));
    MS a(1, 3), b(3, 1);
    a.insert(0, 0, 1); a.insert(0, 1, 1); a.insert(0, 2, 1);
    b.insert(0, 0, 2); b.insert(1, 0, 3); b.insert(2, 0, 4);
    a.lock();
    b.lock();
    EXPECT_DOUBLE_EQ((a * b).get(0, 0), 9.0);
    MS bad(2, 2);
    bad.lock();
    EXPECT_THROW(A * bad, std::invalid_argument);
}

// tests/serial/transpose_tests.cpp:42-178
TEST(Transpose, EntriesMoveAndDoubleTransposeRoundTrips) {
    MS m(3, 4);
    m.insert(0, 0, 1.0);
    m.insert(0, 3, 2.0);
    m.insert(2, 1, 3.0);
    m.lock();
    auto out = ~m;
    EXPECT_EQ(out.n_rows(), 4u);
    EXPECT_EQ(out.n_cols(), 3u);
    EXPECT_DOUBLE_EQ(out.get(0, 0), 1.0);
    EXPECT_DOUBLE_EQ(out.get(3, 0), 2.0);
    EXPECT_DOUBLE_EQ(out.get(1, 2), 3.0);
    EXPECT_DOUBLE_EQ(out.get(2, 0), 0.0);
    auto back = spira::serial::algorithms::transpose(out);
    EXPECT_DOUBLE_EQ(back.get(0, 3), 2.0);
    EXPECT_DOUBLE_EQ(back.get(2, 1), 3.0);
    MS sq(2, 2);
    sq.insert(0, 1, 5.0);
    spira::serial::algorithms::transpose_itself(sq);
    EXPECT_TRUE(sq.is_open());
    EXPECT_DOUBLE_EQ(sq.get(1, 0), 5.0);
    MS rect(2, 3);
    EXPECT_THROW(spira::serial::algorithms::transpose_itself(rect), std::logic_error);
}

// tests/parallel/parallel_matrix_tests.cpp:341-447 (SpMV vs dense, streaming loop)
TEST(ParallelMatrix, FillLockSpmvOpenCycle) {
    using PM = spira::parallel::parallel_matrix<SoA, uint32_t, double>;
    PM pm(100, 80, 3);
    pm.parallel_fill([](auto &rows, std::size_t rs, std::size_t re, std::size_t) {
        for (std::size_t r = rs; r < re; ++r)
            for (uint32_t c = (uint32_t)(r % 7); c < 80; c += 11) rows[r - rs].insert(c, 0.5 * (double)(r + c));
    });
    pm.lock();
    std::vector<double> x(80), y(100);
    for (int i = 0; i < 80; ++i) x[i] = 1.0 / (1 + i);
    for (int cycle = 0; cycle < 3; ++cycle) {
        spira::parallel::algorithms::spmv(pm, x, y);
        for (std::size_t r = 0; r < 100; ++r) {
            double ref = 0;
            for (uint32_t c = 0; c < 80; ++c) ref += pm.get(r, c) * x[c];
            EXPECT_NEAR(y[r], ref, 1e-12 * (1 + std::fabs(ref)));
        }
        pm.open();
        pm.insert((std::size_t)(cycle * 7), 3, 42.0);
        pm.lock();
    }
    EXPECT_DOUBLE_EQ(pm.get(7, 3), 42.0);
    auto T = spira::parallel::algorithms::transpose(pm);
    EXPECT_DOUBLE_EQ(T.get(3, 14), 42.0);
    auto C = spira::parallel::algorithms::spgemm(pm, T);
    EXPECT_EQ(C.n_rows(), 100u);
    pm.rebalance();
    std::size_t covered = 0;
    for (std::size_t t = 0; t < pm.n_threads(); ++t) covered += pm.partition_at(t).size();
    EXPECT_EQ(covered, 100u);
}

// tests/parallel/partition_tests.cpp:16-184 (boundary contract)
TEST(Partition, BoundariesContract) {
    std::vector<std::size_t> nnz = {10, 0, 0, 10, 10, 0, 10};
    auto b = spira::parallel::compute_partition_boundaries(nnz, 4);
    EXPECT_EQ(b.size(), 5u);
    EXPECT_EQ(b.front(), 0u);
    EXPECT_EQ(b.back(), 7u);
    for (std::size_t t = 0; t + 1 < b.size(); ++t) EXPECT_TRUE(b[t] <= b[t + 1]);
    auto z = spira::parallel::compute_partition_boundaries(std::vector<std::size_t>(8, 0), 4);
    EXPECT_EQ(z[1], 2u);
    EXPECT_EQ(z[3], 6u);
}

// tests/serial/matrix_addition_tests.cpp:152-217
TEST(MatrixAddition, ThrowsOnShapeMismatch) {
    MA A(2, 3);
    MA B(3, 2);
    EXPECT_THROW(spira::serial::algorithms::MatrixAddition(A, B), std::invalid_argument);
}

TEST(MatrixAddition, AddsMatricesElementwise_Sparse) {
    MA A(3, 4);
    MA B(3, 4);
    A.insert(0, 0, 1.0);
    A.insert(0, 3, 2.0);
    A.insert(2, 1, 3.0);
    B.insert(0, 0, 10.0);
    B.insert(1, 2, 20.0);
    B.insert(2, 1, -3.0);
    A.lock();
    B.lock();
    auto C = spira::serial::algorithms::MatrixAddition(A, B);
    auto [r, c] = C.shape();
    EXPECT_EQ(r, 3u);
    EXPECT_EQ(c, 4u);
    EXPECT_EQ(C.get(0, 0), 11.0);
    EXPECT_EQ(C.get(0, 3), 2.0);
    EXPECT_EQ(C.get(1, 2), 20.0);
    EXPECT_EQ(C.get(2, 1), 0.0);
    EXPECT_FALSE(C.contains(2, 1));  // the zero sum is dropped
    EXPECT_EQ(C.get(2, 3), 0.0);
    EXPECT_EQ(A.get(0, 0), 1.0);
    EXPECT_EQ(B.get(0, 0), 10.0);
    EXPECT_EQ(A.get(2, 1), 3.0);
    EXPECT_EQ(B.get(2, 1), -3.0);
}

TEST(MatrixAddition, ZeroMatrix_AdditionKeepsOriginal) {
    MA A(2, 2);
    MA Z(2, 2);
    A.insert(0, 1, 7.0);
    A.insert(1, 0, 9.0);
    A.lock();
    Z.lock();
    auto C = spira::serial::algorithms::MatrixAddition(A, Z);
    EXPECT_EQ(C.get(0, 1), 7.0);
    EXPECT_EQ(C.get(1, 0), 9.0);
    EXPECT_EQ(C.get(0, 0), 0.0);
    EXPECT_EQ(C.get(1, 1), 0.0);
    EXPECT_EQ(C.nnz(), 2u);
}

// matrix_operators.hpp:18-62, 104-140: +, -, +=, -=, * s, / s
TEST(MatrixOperators, AddSubScale) {
    MS A(3, 3), B(3, 3);
    A.insert(0, 0, 1.5);
    A.insert(1, 2, -2.0);
    B.insert(0, 0, 0.5);
    B.insert(2, 1, 4.0);
    A.lock();
    B.lock();
    auto S = A + B;
    auto D = A - B;
    EXPECT_EQ(S.get(0, 0), 2.0);
    EXPECT_EQ(S.get(2, 1), 4.0);
    EXPECT_EQ(D.get(0, 0), 1.0);
    EXPECT_EQ(D.get(2, 1), -4.0);
    EXPECT_EQ(D.get(1, 2), -2.0);
    auto Z = A - A;
    EXPECT_EQ(Z.nnz(), 0u);
    auto T = A * 2.0;
    EXPECT_EQ(T.get(1, 2), -4.0);
    auto H = A / 4.0;
    EXPECT_EQ(H.get(0, 0), 0.375);
    EXPECT_THROW(A / 0.0, std::domain_error);
    MS E(3, 4);
    E.lock();
    EXPECT_THROW(A + E, std::invalid_argument);
    A += B;
    EXPECT_EQ(A.get(0, 0), 2.0);
    A -= B;
    EXPECT_EQ(A.get(0, 0), 1.5);
    EXPECT_FALSE(A.contains(2, 1));
}

// tests/serial/scalar_tests.cpp:30-117
TEST(Scalers, MultiplicationScaler_ScalesExistingEntries) {
    MA m(3, 4);
    m.insert(0, 0, 1.5);
    m.insert(0, 3, -2.0);
    m.insert(2, 1, 4.0);
    spira::serial::algorithms::multiplication_scaler(m, 3.0);
    EXPECT_NEAR(m.get(0, 0), 4.5, 1e-12);
    EXPECT_NEAR(m.get(0, 3), -6.0, 1e-12);
    EXPECT_NEAR(m.get(2, 1), 12.0, 1e-12);
    EXPECT_NEAR(m.get(1, 1), 0.0, 1e-12);
    EXPECT_NEAR(m.get(2, 3), 0.0, 1e-12);
}

TEST(Scalers, DivisionScaler_ScalesExistingEntries) {
    MA m(2, 3);
    m.insert(0, 2, 10.0);
    m.insert(1, 0, -6.0);
    spira::serial::algorithms::division_scaler(m, 2.0);
    EXPECT_NEAR(m.get(0, 2), 5.0, 1e-12);
    EXPECT_NEAR(m.get(1, 0), -3.0, 1e-12);
    EXPECT_NEAR(m.get(0, 0), 0.0, 1e-12);
}

TEST(Scalers, MultiplyThenDivide_ReturnsOriginal_ForNonZeroScaler) {
    MA m(3, 3);
    m.insert(0, 1, 1.25);
    m.insert(2, 2, -9.0);
    m.insert(1, 0, 0.5);
    const double a01 = m.get(0, 1), a22 = m.get(2, 2), a10 = m.get(1, 0);
    spira::serial::algorithms::multiplication_scaler(m, 7.0);
    spira::serial::algorithms::division_scaler(m, 7.0);
    EXPECT_NEAR(m.get(0, 1), a01, 1e-12);
    EXPECT_NEAR(m.get(2, 2), a22, 1e-12);
    EXPECT_NEAR(m.get(1, 0), a10, 1e-12);
    EXPECT_NEAR(m.get(0, 0), 0.0, 1e-12);
}

TEST(Scalers, MultiplyByZero_MakesEntriesZero) {
    MA m(2, 2);
    m.insert(0, 0, 3.0);
    m.insert(1, 1, -4.0);
    spira::serial::algorithms::multiplication_scaler(m, 0.0);
    EXPECT_NEAR(m.get(0, 0), 0.0, 1e-12);
    EXPECT_NEAR(m.get(1, 1), 0.0, 1e-12);
}

TEST(Scalers, DivisionByZero_Behavior) {
    MA m(1, 3);
    m.insert(0, 1, 2.0);
    EXPECT_THROW(spira::serial::algorithms::division_scaler(m, 0.0), std::domain_error);
}

// In place on a re-opened matrix: the committed values are scaled on the
// device and survive the next lock; a staged insert at a committed position
// is overridden by the scaled committed value (it was staged before it).
TEST(Scalers, InPlaceAfterLock_ScalesCommittedValues) {
    MS m(3, 3);
    m.insert(0, 0, 2.0);
    m.insert(1, 1, 3.0);
    m.lock();
    m.open();
    m.insert(1, 1, 100.0);
    m.insert(2, 2, 5.0);
    spira::serial::algorithms::multiplication_scaler(m, 0.5);
    m.lock();
    EXPECT_EQ(m.get(0, 0), 1.0);
    EXPECT_EQ(m.get(1, 1), 1.5);
    EXPECT_EQ(m.get(2, 2), 5.0);
    MS out(1, 1);
    spira::serial::algorithms::multiplication_scaler(m, out, 4.0);
    EXPECT_EQ(out.get(1, 1), 6.0);
    EXPECT_EQ(out.nnz(), 3u);
}

// tests/serial/accumulate_algo_tests.cpp:26-160
TEST(Accumulate, SingleRowAndWholeMatrix) {
    using namespace spira::serial::algorithms;
    MA empty(3, 5);
    EXPECT_DOUBLE_EQ(accumulate(empty, 0), 0.0);
    EXPECT_THROW(accumulate(empty, 3), std::out_of_range);
    EXPECT_THROW(accumulate(empty, 100), std::out_of_range);
    auto z = accumulate(empty);
    EXPECT_EQ(z.size(), 3u);
    MA mat(3, 5);
    mat.insert(0, 0, 1.0);
    mat.insert(0, 1, 2.0);
    mat.insert(1, 0, 10.0);
    mat.insert(2, 0, 100.0);
    mat.insert(2, 1, 200.0);
    mat.insert(2, 2, 300.0);
    auto open_r = accumulate(mat);
    EXPECT_DOUBLE_EQ(open_r[0], 3.0);
    EXPECT_DOUBLE_EQ(open_r[1], 10.0);
    EXPECT_DOUBLE_EQ(open_r[2], 600.0);
    mat.lock();
    auto locked_r = accumulate(mat);
    for (int i = 0; i < 3; ++i) EXPECT_DOUBLE_EQ(open_r[i], locked_r[i]);
    MA ow(1, 5);
    ow.insert(0, 0, 10.0);
    ow.insert(0, 0, 25.0);
    EXPECT_DOUBLE_EQ(accumulate(ow, 0), 25.0);
    ow.lock();
    EXPECT_DOUBLE_EQ(accumulate(ow, 0), 25.0);
    // open after a lock: staged entries shadow committed ones
    ow.open();
    ow.insert(0, 0, 1.0);
    ow.insert(0, 4, 2.0);
    EXPECT_DOUBLE_EQ(accumulate(ow, 0), 3.0);
    MA canc(1, 5);
    canc.insert(0, 0, -3.0);
    canc.insert(0, 1, 5.0);
    canc.insert(0, 2, -2.0);
    EXPECT_DOUBLE_EQ(accumulate(canc, 0), 0.0);
}

// parallel/algorithms/matrix_addition.hpp, scalars.hpp, accumulate.hpp and
// parallel_matrix::rebalance
TEST(ParallelAlgorithms, AdditionScalersAccumulateRebalance) {
    using PM = spira::parallel::parallel_matrix<SoA, uint32_t, double>;
    PM A(100, 100, 4), B(100, 100, 4), C3(100, 100, 3);
    for (uint32_t r = 0; r < 100; ++r) {
        A.insert(r, r, 1.0 + r);
        if (r < 10)
            for (uint32_t c = 0; c < 50; ++c) B.insert(r, c, 0.5);
    }
    A.lock();
    B.lock();
    C3.lock();
    EXPECT_THROW(spira::parallel::algorithms::MatrixAddition(A, C3), std::invalid_argument);
    auto S = spira::parallel::algorithms::MatrixAddition(A, B);
    EXPECT_EQ(S.get(3, 3), 4.5);
    EXPECT_EQ(S.get(3, 4), 0.5);
    EXPECT_EQ(S.get(50, 50), 51.0);
    EXPECT_EQ(S.nnz(), 100u + 500u - 10u);
    auto acc = spira::parallel::algorithms::accumulate(S);
    EXPECT_DOUBLE_EQ(acc[0], 1.0 + 49 * 0.5 + 0.5);
    EXPECT_DOUBLE_EQ(spira::parallel::algorithms::accumulate(S, 99), 100.0);
    PM out(100, 100, 4);
    spira::parallel::algorithms::multiplication_scaler(S, out, 2.0);
    EXPECT_EQ(out.get(50, 50), 102.0);
    EXPECT_THROW(spira::parallel::algorithms::division_scaler(S, out, 0.0), std::domain_error);
    S.rebalance();  // nnz-balanced on the device: the 10 dense rows get a partition of their own
    auto p0 = S.partition_at(0);
    EXPECT_EQ(p0.row_start, 0u);
    EXPECT_TRUE(p0.row_end <= 10u);
}

int main() {
    int n = 0;
    for (auto &c : registry()) {
        g_case_failed = false;
        try {
            c.fn();
        } catch (const std::exception &e) {
            std::printf("  uncaught exception: %s\n", e.what());
            g_case_failed = true;
        }
        std::printf("[%s] %s\n", g_case_failed ? "FAIL" : " OK ", c.name);
        g_fail += g_case_failed;
        ++n;
    }
    std::printf("%d tests, %d failed\n", n, g_fail);
    return g_fail;
}
