// test_qr_tall_fat_gpu.cpp — the sequence of the reference's QR tests
// (tests/test_qr_tall.cpp and tests/test_qr_fat.cpp) run through the GB300
// drop-in header <rnp_gpu/QR.hpp>: Factor, MultQ in all four side/trans
// combinations, GenerateQ, and the residuals those tests print, here
// asserted (each in units of m*n*eps, as rsnrm in test_qr_tall.cpp:11).
// Exit status 0 when every residual is at most 10.
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/rnp_gpu/QR.hpp"

template <typename T> struct Real { typedef T type; };
template <typename R> struct Real<std::complex<R> > { typedef R type; };
template <typename T> T conj_(T v) { return v; }
template <typename R> std::complex<R> conj_(std::complex<R> v) { return std::conj(v); }
template <typename T> double eps_() { return (double)std::numeric_limits<typename Real<T>::type>::epsilon(); }

static unsigned long long g_state = 0x1234567ULL;
static double urand() {  // deterministic uniform [-1, 1)
    g_state = g_state * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(g_state >> 11) / 9007199254740992.0 * 2.0 - 1.0;
}
template <typename T> T rnd();
template <> float rnd<float>() { return (float)urand(); }
template <> double rnd<double>() { return urand(); }
template <> std::complex<float> rnd<std::complex<float> >() { float a = (float)urand(); return std::complex<float>(a, (float)urand()); }
template <> std::complex<double> rnd<std::complex<double> >() { double a = urand(); return std::complex<double>(a, urand()); }

template <typename T> struct Dev {
    T *p = nullptr;
    size_t n;
    explicit Dev(size_t count) : n(count) { cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)); }
    ~Dev() { cudaFree(p); }
    void put(const std::vector<T> &h) { cudaMemcpy(p, h.data(), n * sizeof(T), cudaMemcpyHostToDevice); }
    std::vector<T> get() const {
        std::vector<T> h(n);
        cudaDeviceSynchronize();
        cudaMemcpy(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost);
        return h;
    }
};

static int g_fail = 0;
static void report(const char *what, double v) {
    std::printf("  %-28s %.3f\n", what, v);
    if (!(v <= 10.0)) g_fail = 1;
}

template <typename T> void test_qr(size_t m, size_t n) {
    std::printf("%s %zux%zu\n", sizeof(typename Real<T>::type) == 8 ? "double" : "float", m, n);
    const double rsnrm = 1.0 / ((double)(m * n) * eps_<T>());
    const size_t k = std::min(m, n);
    std::vector<T> A(m * n);
    for (auto &v : A) v = rnd<T>();
    Dev<T> dA(m * n), dtau(std::max(m, n)), dB(m * std::max(m, n));
    dA.put(A);
    size_t lwork = 0;
    RNP::LA::QR::Factor(m, n, dA.p, m, dtau.p, &lwork, (T *)nullptr);
    Dev<T> dwork(lwork);
    RNP::LA::QR::Factor(m, n, dA.p, m, dtau.p, &lwork, dwork.p);
    std::vector<T> Afac = dA.get();

    // Q^H A: its upper triangle must be R (test_qr_tall.cpp:43-63)
    std::vector<T> B(A);
    B.resize(m * std::max(m, n));
    dB.put(B);
    size_t lw2 = 0;
    RNP::LA::QR::MultQ("L", "C", m, n, k, dA.p, m, dtau.p, dB.p, m, &lw2, (T *)nullptr);
    Dev<T> dw2(lw2);
    RNP::LA::QR::MultQ("L", "C", m, n, k, dA.p, m, dtau.p, dB.p, m, &lw2, dw2.p);
    B = dB.get();
    double sum = 0;
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i <= std::min(j, m - 1); ++i) sum += std::abs(Afac[i + j * m] - B[i + j * m]);
    report("R norm-1 error", sum * rsnrm);

    // Q R recovers A (test_qr_tall.cpp:65-88)
    std::fill(B.begin(), B.end(), T(0));
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i <= std::min(j, m - 1); ++i) B[i + j * m] = Afac[i + j * m];
    dB.put(B);
    RNP::LA::QR::MultQ("L", "N", m, n, k, dA.p, m, dtau.p, dB.p, m, &lw2, dw2.p);
    B = dB.get();
    sum = 0;
    for (size_t i = 0; i < m * n; ++i) sum += std::abs(A[i] - B[i]);
    report("(A - Q*R) norm-1 error", sum * rsnrm);

    // A^H Q = R^H and R^H Q^H = A^H from the right (test_qr_tall.cpp:90-136)
    size_t lw3 = 0;
    RNP::LA::QR::MultQ("R", "N", n, m, k, dA.p, m, dtau.p, dB.p, n, &lw3, (T *)nullptr);
    Dev<T> dw3(lw3);
    for (size_t j = 0; j < m; ++j)
        for (size_t i = 0; i < n; ++i) B[i + j * n] = conj_(A[j + i * m]);
    dB.put(B);
    RNP::LA::QR::MultQ("R", "N", n, m, k, dA.p, m, dtau.p, dB.p, n, &lw3, dw3.p);
    B = dB.get();
    sum = 0;
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i < std::min(j + 1, m); ++i) sum += std::abs(Afac[i + j * m] - conj_(B[j + i * n]));
    report("R' norm-1 error", sum * rsnrm);
    std::fill(B.begin(), B.end(), T(0));
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i < std::min(j + 1, m); ++i) B[j + i * n] = conj_(Afac[i + j * m]);
    dB.put(B);
    RNP::LA::QR::MultQ("R", "C", n, m, k, dA.p, m, dtau.p, dB.p, n, &lw3, dw3.p);
    B = dB.get();
    sum = 0;
    for (size_t j = 0; j < m; ++j)
        for (size_t i = 0; i < n; ++i) sum += std::abs(conj_(A[j + i * m]) - B[i + j * n]);
    report("(A' - R'*Q') norm-1 error", sum * rsnrm);

    // GenerateQ, Q^H Q = I and Q R = A (test_qr_tall.cpp:138-200)
    const size_t nq = m >= n ? n : m;
    Dev<T> dQ(m * nq);
    cudaMemcpy(dQ.p, dA.p, m * nq * sizeof(T), cudaMemcpyDeviceToDevice);
    size_t lw4 = 0;
    RNP::LA::QR::GenerateQ(m, nq, k, dQ.p, m, dtau.p, &lw4, (T *)nullptr);
    Dev<T> dw4(lw4);
    RNP::LA::QR::GenerateQ(m, nq, k, dQ.p, m, dtau.p, &lw4, dw4.p);
    std::vector<T> Q = dQ.get();
    sum = 0;
    for (size_t j = 0; j < nq; ++j)
        for (size_t i = 0; i < nq; ++i) {
            T s(0);
            for (size_t l = 0; l < m; ++l) s += conj_(Q[l + i * m]) * Q[l + j * m];
            sum += std::abs(s - (i == j ? T(1) : T(0)));
        }
    report("(Q'*Q - I) norm-1 error", sum * rsnrm);
    sum = 0;
    for (size_t j = 0; j < n; ++j)
        for (size_t i = 0; i < m; ++i) {
            T s(0);
            for (size_t l = 0; l <= std::min(j, nq - 1); ++l) s += Q[i + l * m] * Afac[l + j * m];
            sum += std::abs(A[i + j * m] - s);
        }
    report("(A - Q*R) via GenerateQ", sum * rsnrm);
    if (RNP::LA::QR::GPUStatus() != 0) g_fail = 1;
}

int main() {
    // the reference tests' sizes (test_qr_tall.cpp:230-232, test_qr_fat.cpp:214-216)
    test_qr<double>(170, 160);
    test_qr<std::complex<double> >(170, 160);
    test_qr<double>(166, 170);
    test_qr<std::complex<double> >(166, 170);
    test_qr<float>(170, 160);
    test_qr<std::complex<float> >(166, 170);
    std::printf(g_fail ? "FAILED\n" : "OK\n");
    return g_fail;
}
