// refdump -- runs the reference's own host code (compiled from its sources with the
// single-rank MPI and host-only OCCA stand-ins in shim/) and writes its outputs as
// raw little-endian arrays, for the golden fixtures of the test suite.
// Test infrastructure only.
//
//   refdump ogs <nx> <ny> <nz> <p> <perm_seed> <qseed> <outdir>
//       mesh_t on an nx*ny*nz hex box (meshSetup.cpp), optional element-slot
//       permutation of its global ids, ogs_t::Setup(Signed, Auto, unique=true), then
//       the host overloads of GatherScatter(Add, Sym), Gather(Add, Trans),
//       Gather(Add, NoTrans) and Scatter(NoTrans); also the row of every local
//       index (Scatter of the row numbers) and the ids after Setup.
//   refdump ogsmr <size> <nx> <ny> <nz> <p> <qseed> <outdir>
//       the same on `size` ranks (forked processes meeting through the MPI
//       stand-in), each holding an nx*ny*nz box: per rank r, files r<r>_*.bin with
//       the box ids (mesh_t, unsigned), the ids after the mesh's ogs Setup (signed),
//       the counts of a Pairwise handle built on those signed ids, and its
//       GatherScatter (Sym / NoTrans / Trans, Add; Sym, Max), Gather (Trans /
//       NoTrans / Sym, Add) and Scatter (NoTrans / Trans / Sym) on seeded values.
//   refdump bs <N> <seed> <outdir>
//       the BS1-BS5 OKL kernels translated for OCCA Serial execution (okl2cpp.py)
//       on seeded inputs.
#include <sys/wait.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mesh.hpp"

using namespace libp;

namespace {

uint64_t splitmix64(uint64_t* st) {
  uint64_t z = (*st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void uniform(size_t n, uint64_t seed, double* x) {
  uint64_t st = seed;
  for (size_t i = 0; i < n; ++i) {
    const double u = (double)(splitmix64(&st) >> 11) * 0x1.0p-53;
    x[i] = 2.0 * u - 1.0;
  }
}

template <typename T>
void dump(const std::string& dir, const std::string& name, const T* p, size_t n) {
  const std::string path = dir + "/" + name + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::perror(path.c_str());
    std::exit(1);
  }
  std::fwrite(p, sizeof(T), n, f);
  std::fclose(f);
}

class refSettings_t : public settings_t {
 public:
  refSettings_t(int argc, char** argv, comm_t c) : settings_t(c) {
    platformAddSettings(*this);
    meshAddSettings(*this);
    newSetting("-v", "--verbose", "VERBOSE", "FALSE", "Enable verbose output",
               {"TRUE", "FALSE"});
    parseSettings(argc, argv);
  }
};

int run_ogs(int argc, char** argv) {
  if (argc < 9) return 2;
  const std::string nx = argv[2], ny = argv[3], nz = argv[4], p = argv[5];
  const uint64_t perm_seed = std::strtoull(argv[6], nullptr, 10);
  const uint64_t qseed = std::strtoull(argv[7], nullptr, 10);
  const std::string out = argv[8];

  std::vector<std::string> args = {"refdump", "-m", "Serial", "-e", "Hex", "-nx", nx,
                                   "-ny", ny, "-nz", nz, "-p", p};
  std::vector<char*> av;
  for (auto& s : args) av.push_back(const_cast<char*>(s.c_str()));
  comm_t comm(Comm::World().Dup());
  refSettings_t settings((int)av.size(), av.data(), comm);
  platform_t platform(settings);
  mesh_t mesh(platform, settings, comm);

  const dlong N = mesh.Nelements * mesh.Np;
  ogs::ogs_t* ogs = &mesh.ogs;
  ogs::ogs_t permuted;
  memory<hlong> ids = mesh.globalIds;
  if (perm_seed != 0) {
    // move lexicographic element e to slot perm[e] (seeded Fisher-Yates, SplitMix64)
    const dlong E = mesh.Nelements, Np = mesh.Np;
    std::vector<dlong> slot(E);
    for (dlong e = 0; e < E; ++e) slot[e] = e;
    uint64_t st = perm_seed;
    for (dlong i = E - 1; i > 0; --i) {
      const dlong j = (dlong)(splitmix64(&st) % (uint64_t)(i + 1));
      std::swap(slot[i], slot[j]);
    }
    // unsigned ids of the lexicographic mesh, then permute element blocks
    memory<hlong> absIds(N);
    for (dlong l = 0; l < N; ++l) absIds[l] = std::abs(mesh.globalIds[l]);
    ids.malloc(N);
    for (dlong e = 0; e < E; ++e)
      for (dlong n = 0; n < Np; ++n) ids[slot[e] * Np + n] = absIds[e * Np + n];
    permuted.Setup(N, ids, comm, ogs::Signed, ogs::Auto, true, false, platform);
    ogs = &permuted;
  }
  const dlong Ng = ogs->Ngather;
  std::printf("N=%d Ngather=%d NgatherGlobal=%lld\n", N, Ng, (long long)ogs->NgatherGlobal);

  dump(out, "ids", ids.ptr(), N);

  // row of every local index
  memory<long long int> rows(Ng), rowOf(N, -1);
  for (dlong r = 0; r < Ng; ++r) rows[r] = r;
  ogs->Scatter(rowOf, rows, 1, ogs::NoTrans);
  dump(out, "row_of", rowOf.ptr(), N);

  memory<double> q(N), gq(Ng), g(Ng), qs(N, 0.0);
  uniform(N, qseed, q.ptr());
  uniform(Ng, qseed + 1, g.ptr());
  dump(out, "q", q.ptr(), N);

  ogs->Gather(gq, q, 1, ogs::Add, ogs::Trans);
  dump(out, "gather_trans", gq.ptr(), Ng);
  ogs->Gather(gq, q, 1, ogs::Add, ogs::NoTrans);
  dump(out, "gather_notrans", gq.ptr(), Ng);
  ogs->Scatter(qs, g, 1, ogs::NoTrans);
  dump(out, "scatter_notrans", qs.ptr(), N);
  memory<double> qgs = q.clone();
  ogs->GatherScatter(qgs, 1, ogs::Add, ogs::Sym);
  dump(out, "gs_sym", qgs.ptr(), N);
  return 0;
}

int ogsmr_rank(const std::string& nx, const std::string& ny, const std::string& nz,
               const std::string& p, uint64_t qseed, const std::string& out) {
  std::vector<std::string> args = {"refdump", "-m", "Serial", "-e", "Hex", "-nx", nx,
                                   "-ny", ny, "-nz", nz, "-p", p};
  std::vector<char*> av;
  for (auto& s : args) av.push_back(const_cast<char*>(s.c_str()));
  comm_t comm(Comm::World().Dup());
  const int rank = comm.rank();
  refSettings_t settings((int)av.size(), av.data(), comm);
  platform_t platform(settings);
  mesh_t mesh(platform, settings, comm);
  const dlong N = mesh.Nelements * mesh.Np;
  const std::string pre = out + "/r" + std::to_string(rank) + "_";
  auto put = [&](const std::string& name, auto* ptr, size_t n) { dump(out, "r" + std::to_string(rank) + "_" + name, ptr, n); };
  (void)pre;

  // the mesh's own handle (Auto, unique) flagged one owner per group
  memory<hlong> ids = mesh.globalIds.clone();
  memory<hlong> absIds(N);
  for (dlong l = 0; l < N; ++l) absIds[l] = std::abs(ids[l]);
  put("box_ids", absIds.ptr(), N);
  put("ids", ids.ptr(), N);

  ogs::ogs_t pw;
  pw.Setup(N, ids, comm, ogs::Signed, ogs::Pairwise, false, false, platform);
  const long long counts[8] = {pw.N, pw.NlocalP, pw.NlocalT, pw.NhaloP, pw.NhaloT, pw.Ngather,
                               (long long)pw.NgatherGlobal, pw.gather_defined ? 1 : 0};
  put("counts", counts, 8);

  const dlong G = pw.NlocalT + pw.NhaloT;
  memory<double> q(N), g(G > 0 ? G : 1);
  uniform(N, qseed + 1000 * rank, q.ptr());
  uniform(G, qseed + 1000 * rank + 1, g.ptr());
  put("q", q.ptr(), N);
  put("g", g.ptr(), G);
  const ogs::Transpose modes[3] = {ogs::Sym, ogs::NoTrans, ogs::Trans};
  const char* names[3] = {"sym", "notrans", "trans"};
  for (int m = 0; m < 3; ++m) {
    memory<double> v = q.clone();
    pw.GatherScatter(v, 1, ogs::Add, modes[m]);
    put(std::string("gs_") + names[m], v.ptr(), N);
    memory<double> gv(G > 0 ? G : 1);
    for (dlong i = 0; i < G; ++i) gv[i] = 0.0;
    pw.Gather(gv, q, 1, ogs::Add, modes[m]);
    put(std::string("gather_") + names[m], gv.ptr(), G);
    memory<double> vs(N);
    for (dlong i = 0; i < N; ++i) vs[i] = 0.0;
    pw.Scatter(vs, g, 1, modes[m]);
    put(std::string("scatter_") + names[m], vs.ptr(), N);
  }
  memory<double> vm = q.clone();
  pw.GatherScatter(vm, 1, ogs::Max, ogs::Sym);
  put("gs_sym_max", vm.ptr(), N);
  return 0;
}

int run_ogsmr(int argc, char** argv) {
  if (argc < 9) return 2;
  const int size = std::atoi(argv[2]);
  const std::string nx = argv[3], ny = argv[4], nz = argv[5], p = argv[6];
  const uint64_t qseed = std::strtoull(argv[7], nullptr, 10);
  const std::string out = argv[8];
  if (sp_mpi_start(size, (size_t)256 << 20, (size_t)64 << 20)) return 1;
  std::vector<pid_t> kids;
  for (int r = 0; r < size; ++r) {
    const pid_t pid = fork();
    if (pid < 0) return 1;
    if (pid == 0) {
      sp_mpi_set_rank(r);
      std::fflush(stdout);
      _exit(ogsmr_rank(nx, ny, nz, p, qseed, out));
    }
    kids.push_back(pid);
  }
  int rc = 0;
  for (pid_t k : kids) {
    int st = 0;
    waitpid(k, &st, 0);
    if (!WIFEXITED(st) || WEXITSTATUS(st) != 0) rc = 1;
  }
  std::printf("ogsmr size=%d rc=%d\n", size, rc);
  return rc;
}

}  // namespace

// BS1-BS5 kernels (OCCA Serial translation of the reference's OKL)
extern "C" {
void bs1(const int N, const double* a, double* b);
void bs2(const int N, const double alpha, const double* x, const double beta, double* y);
void bs3_1_256(const int Nblocks, const int N, const double* a, double* norm);
void bs3_2_256(const int Nblocks, const double* a, double* norm);
void bs4_1_256(const int Nblocks, const int N, const double* a, const double* bb, double* ddot);
void bs4_2_256(const int Nblocks, const double* a, double* ddot);
void bs5_1_1024(const int Nblocks, const int N, const double* Ap, const double alpha, double* r,
                double* rdotr);
void bs5_2_1024(const int Nblocks, const double* a, double* ddot);
void bs5_1_256(const int Nblocks, const int N, const double* Ap, const double alpha, double* r,
               double* rdotr);
void bs5_2_256(const int Nblocks, const double* a, double* ddot);
}

static int run_bs(int argc, char** argv) {
  if (argc < 5) return 2;
  const int N = std::atoi(argv[2]);
  const uint64_t seed = std::strtoull(argv[3], nullptr, 10);
  const std::string out = argv[4];
  std::vector<double> a(N), b(N), y(N), r(N), tmp(1024), res(1);
  uniform(N, seed, a.data());
  uniform(N, seed + 1, b.data());
  const double alpha = -0.7353, beta = 0.4142;
  bs1(N, a.data(), y.data());
  dump(out, "bs1", y.data(), N);
  y = b;
  bs2(N, alpha, a.data(), beta, y.data());
  dump(out, "bs2", y.data(), N);
  auto nb = [N](int bsz) { int n = (N + bsz - 1) / bsz; return n > bsz ? bsz : (n < 1 ? 1 : n); };
  bs3_1_256(nb(256), N, a.data(), tmp.data());
  bs3_2_256(nb(256), tmp.data(), res.data());
  dump(out, "bs3_partial", tmp.data(), nb(256));
  dump(out, "bs3", res.data(), 1);
  bs4_1_256(nb(256), N, a.data(), b.data(), tmp.data());
  bs4_2_256(nb(256), tmp.data(), res.data());
  dump(out, "bs4_partial", tmp.data(), nb(256));
  dump(out, "bs4", res.data(), 1);
  r = b;
  bs5_1_1024(nb(1024), N, a.data(), alpha, r.data(), tmp.data());
  bs5_2_1024(nb(1024), tmp.data(), res.data());
  dump(out, "bs5_r", r.data(), N);
  dump(out, "bs5_partial", tmp.data(), nb(1024));
  dump(out, "bs5", res.data(), 1);
  r = b;
  bs5_1_256(nb(256), N, a.data(), alpha, r.data(), tmp.data());
  bs5_2_256(nb(256), tmp.data(), res.data());
  dump(out, "bs5_256", res.data(), 1);
  return 0;
}

int main(int argc, char** argv) {
  Comm::Init(argc, argv);
  int rc = 2;
  if (argc > 1 && std::string(argv[1]) == "ogs") rc = run_ogs(argc, argv);
  else if (argc > 1 && std::string(argv[1]) == "ogsmr") rc = run_ogsmr(argc, argv);
  else if (argc > 1 && std::string(argv[1]) == "bs") rc = run_bs(argc, argv);
  if (rc == 2) std::fprintf(stderr, "usage: refdump ogs nx ny nz p perm_seed qseed outdir | bs N seed outdir\n");
  Comm::Finalize();
  return rc;
}
