// noalloc.cu -- conjugate-gradient solve that allocates nothing.
//
// Some callers cannot let a library allocate device memory: an application whose own memory
// pool owns the whole device (a cudaMalloc from here would fail or fragment it), or an
// embedding whose solve path must not allocate (real-time or certified code that reserves all
// memory up front).  dg_cg_noalloc serves them: the caller passes the matrix (full CRS) and the
// vectors in device memory, and every temporary the solve needs (three work vectors, the
// reduction partials, the validation word and the solver scalars) lives in one file-scope
// static device array of fixed size.  No cudaMalloc, cudaFree, pinned-host or library
// allocation happens on this path.
//
// Limits and sharing:
//  * n <= kNoAllocMaxN rows (the array holds three vectors of that length); larger systems
//    are rejected with DG_ERR_ARG before any device work;
//  * the caller's CRS is checked on the device first (row offsets from 0 to row[n],
//    non-decreasing; columns in [0, n)) and a malformed one is rejected with DG_ERR_MATRIX
//    before any product reads through it;
//  * the array is one per device and every call on that device shares it, keeping the last
//    call's contents; the call clears what must start at zero (reduction ticket, validation
//    word, solver state).  Calls from one process take one process-wide mutex, so calls on
//    different devices also run one at a time; any other device work that touches the array
//    while a call runs would race with it;
//  * the call runs on the library's own per-thread stream and returns after that stream has
//    finished (also on every error path, before the mutex is released); the inputs must
//    already be complete on the device when it is called;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress,
//    with that device current) and caches it, so make that first call before any stream
//    capture begins.
#include <mutex>

#include "krylov.cuh"
#include "matrix.cuh"

namespace dg {
namespace {

constexpr long kNoAllocMaxN = 1L << 20;            // rows
constexpr int kNoAllocMaxGrid = 4096;              // reduction partials
constexpr size_t kVecBytes = sizeof(double) * (size_t)kNoAllocMaxN;
constexpr size_t kOffR = 0, kOffP = kVecBytes, kOffY = 2 * kVecBytes;
constexpr size_t kOffPartials = 3 * kVecBytes;
constexpr size_t kOffPartials2 = kOffPartials + sizeof(double) * kNoAllocMaxGrid;   // update -> direction
constexpr size_t kOffScalars = kOffPartials2 + sizeof(double) * kNoAllocMaxGrid;
constexpr size_t kOffProgress = kOffScalars + ((sizeof(Scalars) + 255) / 256) * 256;
constexpr size_t kOffTicket = kOffProgress + ((sizeof(Progress) + 255) / 256) * 256;
constexpr size_t kOffBad = kOffTicket + 256;         // validation: first malformed row
constexpr size_t kScratchBytes = kOffBad + 256;

// The scratch array: 3 x 8 MiB vectors + partials + state, about 24 MiB per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_noalloc_mutex;
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (looked up once per device).
unsigned char *scratch_for_current_device() {
  int dev = 0;
  DG_CUDA(cudaGetDevice(&dev));
  DG_REQUIRE(dev >= 0 && dev < kMaxDevices, DG_ERR_ARG, "device %d out of range", dev);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    DG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
  }
  return g_scratch_ptr[dev];
}

// Waits for the stream on every exit path, so that no kernel of this call is still running on
// the shared array once the mutex is released.
struct StreamDrain {
  cudaStream_t st;
  ~StreamDrain() { cudaStreamSynchronize(st); }
};

struct RawCrsLauncher {
  CrsOp<double> op;
  int n_, lanes, grid_;
  int n() const { return n_; }
  int grid() const { return grid_; }
  long nnz() const { return 0; }
  template <class XT, class Epi>
  void apply(const XT *x, Scale sc, double sigma, const int *gate, const Epi &epi, RedSlot slot,
             cudaStream_t st) const {
    launch_apply(op, lanes, grid_, n_, x, sc, sigma, gate, epi, slot, st);
  }
};

}  // namespace
}  // namespace dg

using namespace dg;

extern "C" int dg_cg_noalloc(int n, const long *row_dev, const int *col_dev, const double *val_dev, double sigma,
                             const double *b_dev, double *x_dev, double acc, int max_step, int *iters) {
  return guarded([&] {
    require_device();
    DG_REQUIRE(row_dev && col_dev && val_dev && b_dev && x_dev, DG_ERR_ARG, "null argument");
    DG_REQUIRE(n > 0, DG_ERR_ARG, "n must be positive (n=%d)", n);
    DG_REQUIRE(n <= kNoAllocMaxN, DG_ERR_ARG, "n=%d exceeds the allocation-free limit of %ld rows", n, kNoAllocMaxN);
    DG_REQUIRE(max_step >= 1, DG_ERR_ARG, "max_step must be >= 1");
    DG_REQUIRE(is_device_ptr(row_dev) && is_device_ptr(col_dev) && is_device_ptr(val_dev) && is_device_ptr(b_dev) &&
                   is_device_ptr(x_dev),
               DG_ERR_ARG, "dg_cg_noalloc takes device pointers only");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    cudaStream_t st = stream();
    StreamDrain drain{st};
    unsigned char *base = scratch_for_current_device();
    double *r = reinterpret_cast<double *>(base + kOffR);
    double *p = reinterpret_cast<double *>(base + kOffP);
    double *y = reinterpret_cast<double *>(base + kOffY);
    double *partials = reinterpret_cast<double *>(base + kOffPartials);
    double *partials2 = reinterpret_cast<double *>(base + kOffPartials2);
    Scalars *S = reinterpret_cast<Scalars *>(base + kOffScalars);
    Progress *prog = reinterpret_cast<Progress *>(base + kOffProgress);
    unsigned *ticket = reinterpret_cast<unsigned *>(base + kOffTicket);
    int *bad = reinterpret_cast<int *>(base + kOffBad);

    int64_t ends[2];
    DG_CUDA(cudaMemcpyAsync(&ends[0], row_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaMemcpyAsync(&ends[1], row_dev + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(ends[0] == 0 && ends[1] >= 0, DG_ERR_MATRIX, "CRS row offsets must run from 0 to row[n] >= 0");
    // The CRS invariants, checked on the device before any product gathers through the columns.
    const int big = 0x7fffffff;
    int first_bad = 0;
    DG_CUDA(cudaMemcpyAsync(bad, &big, sizeof(int), cudaMemcpyHostToDevice, st));
    launch_validate(reinterpret_cast<const int64_t *>(row_dev), col_dev, n, (long)ends[1], 0, bad, st);
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaMemcpyAsync(&first_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    DG_REQUIRE(first_bad == big, DG_ERR_MATRIX, "row %d has a column outside [0, n) or decreasing offsets", first_bad);
    RawCrsLauncher op;
    op.op = CrsOp<double>{reinterpret_cast<const int64_t *>(row_dev), col_dev, val_dev};
    op.n_ = n;
    choose_shape(n, (long)ends[1], &op.lanes, &op.grid_);
    const int vgrid = vector_grid(n);
    DG_REQUIRE(op.grid_ <= kNoAllocMaxGrid && vgrid <= kNoAllocMaxGrid, DG_ERR_ARG, "grid exceeds the scratch partials");
    const RedSlot slot{partials, ticket};

    // State that must start at zero: the reduction ticket and the solver scalars / progress.
    DG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), st));
    DG_CUDA(cudaMemsetAsync(S, 0, sizeof(Scalars), st));
    DG_CUDA(cudaMemsetAsync(prog, 0, sizeof(Progress), st));

    // x0 normalised (into y), r = b - (M + sigma) x0, p = r; then x <- normalised x0
    // (sml/CONJUGATE_GRADIENT_SYM.c:35-43).
    k_norm2<double><<<vgrid, kThreads, 0, st>>>(x_dev, n, &S->xn2, slot); ::dg::count_launch();
    op.apply(x_dev, Scale::norm2(&S->xn2), sigma, (const int *)nullptr, EpiCgInit{b_dev, y, r, p, S}, slot, st);
    DG_CUDA(cudaMemcpyAsync(x_dev, y, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    const int chunk = 16;
    int done = 0, it = 1;
    while (it < max_step && !done) {
      const int last = std::min(it + chunk - 1, max_step - 1);
      for (; it <= last; ++it) {
        op.apply(p, Scale{}, sigma, &S->done, EpiCgDot{y}, slot, st);
        k_cg_update<<<vgrid, kThreads, 0, st>>>(n, p, y, x_dev, r, S, it, partials, op.grid_, partials2); ::dg::count_launch();
        k_cg_direction<<<vgrid, kThreads, 0, st>>>(n, r, p, S, it, max_step, acc, partials2, vgrid, prog); ::dg::count_launch();
      }
      DG_CUDA(cudaGetLastError());
      DG_CUDA(cudaMemcpyAsync(&done, &S->done, sizeof(int), cudaMemcpyDeviceToHost, st));
      DG_CUDA(cudaStreamSynchronize(st));
    }
    int it_done = max_step;
    DG_CUDA(cudaMemcpyAsync(&it_done, &S->iters, sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    if (iters) *iters = done ? it_done : max_step;
    DG_REQUIRE(done == 1, DG_ERR_NOCONV, "CG did not converge (max step %d)", max_step);
  });
}
