// Drives the C++ drop-in (include/stq_gpu.hpp) the way the reference's app
// does (app/main.cu:82-152): constructBoxes, then run_sweep_sharedqueue with
// KEEP_CPU_OVERLAPS, then run_sweep_multigpu. Reads a mesh from a binary file
// and writes the boxes and both pair lists for the test to compare.
//
//   shim_check <mesh.bin> <out_prefix> once|loop [memlimit_gb]
//   mesh.bin: int64 nV, nE, nF; f64 V0[nV*3]; f64 V1[nV*3]; i32 E[nE*2]; i32 F[nF*3]
//
// once: a single run_sweep_sharedqueue call, exactly as app/main.cu:140-143
//       makes it; tidstart must come back >= N.
// loop: calls while (tidstart < N), freeing the previous call's buffers
//       (built with STQ_GPU_MAX_OVERLAP_SIZE so that the pair buffer overflows
//       and the cutoff is halved).
#define KEEP_CPU_OVERLAPS
#include "stq_gpu.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

// The minimal matrix interface the drop-in needs (Eigen's MatrixXd/MatrixXi
// provide the same rows() / cols() / operator()(i, j)).
template <typename T>
struct Matrix {
  long r = 0, c = 0;
  std::vector<T> v;
  long rows() const { return r; }
  long cols() const { return c; }
  T operator()(long i, long j) const { return v[size_t(i * c + j)]; }
};

template <typename T>
static void read(std::ifstream &in, Matrix<T> &m, long rows, long cols) {
  m.r = rows, m.c = cols, m.v.resize(size_t(rows * cols));
  in.read(reinterpret_cast<char *>(m.v.data()), std::streamsize(sizeof(T) * m.v.size()));
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  std::ifstream in(argv[1], std::ios::binary);
  int64_t n[3];
  in.read(reinterpret_cast<char *>(n), sizeof n);
  Matrix<double> V0, V1;
  Matrix<int> E, F;
  read(in, V0, n[0], 3);
  read(in, V1, n[0], 3);
  read(in, E, n[1], 2);
  read(in, F, n[2], 3);
  if (!in) return 3;
  const std::string out = argv[2];
  const std::string mode = argc > 3 ? argv[3] : "once";
  const int memlimit = argc > 4 ? std::atoi(argv[4]) : 0;
  if (mode != "once" && mode != "loop") return 2;
  try {
    std::vector<stq::gpu::Aabb> boxes;
    stq::gpu::constructBoxes(V0, V1, E, F, boxes);
    {
      std::ofstream f(out + ".boxes", std::ios::binary);
      f.write(reinterpret_cast<const char *>(boxes.data()), std::streamsize(sizeof(stq::gpu::Aabb) * boxes.size()));
    }
    stq::gpu::MemHandler *memhandle = new stq::gpu::MemHandler();
    std::vector<std::pair<int, int>> overlaps;
    int2 *d_overlaps = nullptr;
    int *d_count = nullptr;
    int threads = 0, tidstart = 0, devcount = 1;
    const int N = int(boxes.size());
    stq::gpu::run_sweep_sharedqueue(boxes.data(), memhandle, N, 0, overlaps, d_overlaps, d_count,
                                    threads, tidstart, devcount, memlimit);
    int calls = 1;
    while (mode == "loop" && tidstart < N) {
      cudaFree(d_overlaps);
      cudaFree(d_count);
      stq::gpu::run_sweep_sharedqueue(boxes.data(), memhandle, N, 0, overlaps, d_overlaps, d_count,
                                      threads, tidstart, devcount, memlimit);
      ++calls;
    }
    if (tidstart < N) {
      std::fprintf(stderr, "error: tidstart %d < N %d after %d call(s)\n", tidstart, N, calls);
      return 4;
    }
    int dc = -1;
    cudaMemcpy(&dc, d_count, sizeof(int), cudaMemcpyDeviceToHost);
    {
      std::ofstream f(out + ".stq", std::ios::binary);
      for (auto &p : overlaps) f.write(reinterpret_cast<const char *>(&p), sizeof p);
    }
    std::vector<std::pair<int, int>> plain;
    stq::gpu::run_sweep_multigpu(boxes.data(), N, 0, plain, threads, devcount);
    {
      std::ofstream f(out + ".plain", std::ios::binary);
      for (auto &p : plain) f.write(reinterpret_cast<const char *>(&p), sizeof p);
    }
    std::printf("boxes %d stq_pairs %zu plain_pairs %zu calls %d cutoff %zu last_count %d tidstart %d\n", N,
                overlaps.size(), plain.size(), calls, memhandle->MAX_OVERLAP_CUTOFF, dc, tidstart);
    cudaFree(d_overlaps);
    cudaFree(d_count);
    delete memhandle;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
