// Replacements for the parts of the reference's libs/core that need OCCA's JIT
// device setup or LAPACK, so that the reference's host code can be compiled into
// the test checker.  Written for this checker; not part of the product.
//   * platform_t::DeviceConfig: a host-only "Serial" device (the checker only runs
//     host overloads).
//   * matrixEigenVectors / matrixEigenValues: cyclic Jacobi eigen-solver for the
//     symmetric matrices the mesh code passes (the Jacobi recurrence matrix of
//     JacobiGQ, libs/mesh/meshBasis1D.cpp:195-250).
//   * matrixInverse / matrixRightSolve: Gauss-Jordan elimination with partial pivoting.
// Only node coordinates depend on these, and coordinates only enter tolerance-based
// face matching; the global ids of a box mesh do not depend on their last bits.
// Also the shared state of the MPI stand-in (shim/mpi.h).
#include <sys/mman.h>

#include <cmath>
#include <vector>

#include "platform.hpp"

struct sp_mpi_world* sp_mpi_w = nullptr;
int sp_mpi_rank = 0;
size_t sp_mpi_type_size[4096] = {0, 1, 4, 8, 4, 8};
int sp_mpi_ntypes = 6;
struct sp_mpi_req sp_mpi_reqs[SP_MPI_MAXREQ];
int sp_mpi_ncomms = MPI_COMM_WORLD;

int sp_mpi_start(int size, size_t area_bytes, size_t box_bytes) {
  if (size < 1 || size > SP_MPI_MAXRANKS) return 1;
  const size_t total = sizeof(sp_mpi_world) + (size_t)size * (area_bytes + box_bytes);
  void* p = mmap(nullptr, total, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (p == MAP_FAILED) return 1;
  sp_mpi_world* w = static_cast<sp_mpi_world*>(p);
  w->size = size;
  w->area_bytes = area_bytes;
  w->box_bytes = box_bytes;
  pthread_barrierattr_t ba;
  pthread_barrierattr_init(&ba);
  pthread_barrierattr_setpshared(&ba, PTHREAD_PROCESS_SHARED);
  pthread_barrier_init(&w->bar, &ba, (unsigned)size);
  pthread_mutexattr_t ma;
  pthread_mutexattr_init(&ma);
  pthread_mutexattr_setpshared(&ma, PTHREAD_PROCESS_SHARED);
  pthread_mutex_init(&w->mtx, &ma);
  pthread_condattr_t ca;
  pthread_condattr_init(&ca);
  pthread_condattr_setpshared(&ca, PTHREAD_PROCESS_SHARED);
  pthread_cond_init(&w->cv, &ca);
  for (int r = 0; r < size; ++r) w->box[r].nmsg = w->box[r].live = 0, w->box[r].used = 0;
  sp_mpi_w = w;
  return 0;
}

void sp_mpi_set_rank(int rank) { sp_mpi_rank = rank; }

namespace libp {

void platform_t::DeviceConfig() {
  device.setup(properties_t());
}

static void jacobi_eig(int N, const double* A, double* W, double* V) {
  std::vector<double> a(A, A + (size_t)N * N);
  for (int i = 0; i < N * N; ++i) V[i] = 0.0;
  for (int i = 0; i < N; ++i) V[i * N + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < N; ++p)
      for (int q = p + 1; q < N; ++q) off += a[p * N + q] * a[p * N + q];
    if (off < 1e-300) break;
    for (int p = 0; p < N; ++p)
      for (int q = p + 1; q < N; ++q) {
        const double apq = a[p * N + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a[q * N + q] - a[p * N + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < N; ++k) {  // A <- A J
          const double akp = a[k * N + p], akq = a[k * N + q];
          a[k * N + p] = c * akp - s * akq;
          a[k * N + q] = s * akp + c * akq;
        }
        for (int k = 0; k < N; ++k) {  // A <- J^T A
          const double apk = a[p * N + k], aqk = a[q * N + k];
          a[p * N + k] = c * apk - s * aqk;
          a[q * N + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < N; ++k) {  // V <- V J (columns are eigenvectors)
          const double vkp = V[k * N + p], vkq = V[k * N + q];
          V[k * N + p] = c * vkp - s * vkq;
          V[k * N + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < N; ++i) W[i] = a[i * N + i];
}

void matrixEigenVectors(int N, double* A, double* VR, double* WR, double* WI) {
  jacobi_eig(N, A, WR, VR);
  for (int i = 0; i < N; ++i) WI[i] = 0.0;
}

void matrixEigenVectors(int N, float* A, float* VR, float* WR, float* WI) {
  std::vector<double> a(A, A + (size_t)N * N), v((size_t)N * N), w(N);
  jacobi_eig(N, a.data(), w.data(), v.data());
  for (int i = 0; i < N * N; ++i) VR[i] = (float)v[i];
  for (int i = 0; i < N; ++i) {
    WR[i] = (float)w[i];
    WI[i] = 0.f;
  }
}

void matrixEigenValues(int N, double* A, double* WR, double* WI) {
  std::vector<double> v((size_t)N * N);
  matrixEigenVectors(N, A, v.data(), WR, WI);
}

void matrixEigenValues(int N, float* A, float* WR, float* WI) {
  std::vector<float> v((size_t)N * N);
  matrixEigenVectors(N, A, v.data(), WR, WI);
}

template <typename T>
static void gauss_jordan_inverse(int N, T* A) {
  std::vector<double> a(A, A + (size_t)N * N), inv((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i) inv[i * N + i] = 1.0;
  for (int c = 0; c < N; ++c) {
    int piv = c;
    for (int r = c + 1; r < N; ++r)
      if (std::fabs(a[r * N + c]) > std::fabs(a[piv * N + c])) piv = r;
    LIBP_ABORT("matrixInverse: singular matrix", a[piv * N + c] == 0.0);
    for (int k = 0; k < N; ++k) {
      std::swap(a[c * N + k], a[piv * N + k]);
      std::swap(inv[c * N + k], inv[piv * N + k]);
    }
    const double d = a[c * N + c];
    for (int k = 0; k < N; ++k) {
      a[c * N + k] /= d;
      inv[c * N + k] /= d;
    }
    for (int r = 0; r < N; ++r) {
      if (r == c) continue;
      const double f = a[r * N + c];
      if (f == 0.0) continue;
      for (int k = 0; k < N; ++k) {
        a[r * N + k] -= f * a[c * N + k];
        inv[r * N + k] -= f * inv[c * N + k];
      }
    }
  }
  for (int i = 0; i < N * N; ++i) A[i] = (T)inv[i];
}

void matrixInverse(int N, double* A) { gauss_jordan_inverse(N, A); }
void matrixInverse(int N, float* A) { gauss_jordan_inverse(N, A); }

// C = A / B = A * inv(B), row major; A is NrowsA x NcolsA, B is NrowsB x NcolsB (square).
template <typename T>
static void right_solve(int NrowsA, int NcolsA, T* A, int NrowsB, int NcolsB, T* B, T* C) {
  std::vector<T> binv(B, B + (size_t)NrowsB * NcolsB);
  gauss_jordan_inverse(NrowsB, binv.data());
  for (int i = 0; i < NrowsA; ++i)
    for (int j = 0; j < NcolsB; ++j) {
      double s = 0.0;
      for (int k = 0; k < NcolsA; ++k) s += (double)A[i * NcolsA + k] * binv[k * NcolsB + j];
      C[i * NcolsB + j] = (T)s;
    }
}

void matrixRightSolve(int NrowsA, int NcolsA, double* A, int NrowsB, int NcolsB, double* B,
                      double* C) {
  right_solve(NrowsA, NcolsA, A, NrowsB, NcolsB, B, C);
}
void matrixRightSolve(int NrowsA, int NcolsA, float* A, int NrowsB, int NcolsB, float* B,
                      float* C) {
  right_solve(NrowsA, NcolsA, A, NrowsB, NcolsB, B, C);
}

}  // namespace libp
