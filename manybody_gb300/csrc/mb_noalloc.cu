// mb_op_apply_noalloc: y = H x in reference order without allocating.
//
// Who needs it: mb_op_apply in reference order permutes x into the engine's
// tensor order, applies H and permutes back, through two vector-sized
// scratch buffers that the library cudaMalloc's on first use (plus a
// permutation table).  Some callers cannot let the library allocate: host
// frameworks that own all device memory through their own pool and a fixed
// budget (an ED service next to other resident models), and latency-critical
// loops where cudaMalloc's implicit device synchronisation is not acceptable.
// This entry point takes its scratch from a fixed array compiled into the
// library instead, and computes the basis permutation on the fly.
//
// Limits and rules:
//   * at most kNoAllocMaxDim = 1,048,576 basis states (the scratch array holds
//     two vectors of that many complex128 elements: 32 MiB, plus 512 bytes for
//     the block-floating-point parameters); larger sectors are rejected with
//     MB_ERR_CAPACITY;
//   * the arrays live in the library's device code.  CUDA loads that code
//     into a device lazily (the default since CUDA 12.2), and the first call on
//     a device is what loads it there: that call takes the 32 MiB on that
//     device (held until the process exits), looks up the arrays' device
//     addresses (cudaGetSymbolAddress) and uploads a 9 KB binomial table, with
//     the device current (it must be the operator's device).  Make the first
//     call during set-up, before any stream capture; later calls allocate
//     nothing;
//   * MB_PREC_Q64 operators take the same steps as mb_op_apply on them
//     (conversion to block floating point with the vector's exponent, the
//     integer apply, conversion back), so the results are the same bits;
//   * every call on a device shares the one array: calls whose work overlaps
//     on the GPU (different streams, different host threads) race and corrupt
//     each other's results -- serialise them;
//   * the array keeps the previous call's contents; every element this entry
//     point reads from it is written earlier in the same call, so nothing
//     needs clearing.
#include <cuda_runtime.h>

#include <mutex>

#include "mb_internal.h"
#include "mb_q64.h"

namespace mb {
namespace {

constexpr int64_t kNoAllocMaxDim = int64_t(1) << 20;
constexpr int kNoAllocMaxDevices = 64;

// Two tensor-order vectors (x permuted, H x before the inverse permutation).
static __device__ __align__(256) double2 g_noalloc_scratch[2 * kNoAllocMaxDim];
// The block-floating-point parameters of a Q64 call: QParams, then 4 ints
// (largest biased exponent, the vector's exponent).
constexpr size_t kNoAllocIntsAt = 384;
static_assert(sizeof(QParams) <= kNoAllocIntsAt, "QParams outgrew its slot");
static __device__ __align__(256) unsigned char g_noalloc_small[512];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
void* g_noalloc_small_ptr[kNoAllocMaxDevices] = {};

// Device addresses of the two arrays on device `dev` (current), looked up once.
void* noalloc_scratch(int dev, void** small) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    void* q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    MB_REQUIRE(e == cudaSuccess && p, MB_ERR_CUDA,
               std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&q, g_noalloc_small);
    MB_REQUIRE(e == cudaSuccess && q, MB_ERR_CUDA,
               std::string("cudaGetSymbolAddress(g_noalloc_small): ") + cudaGetErrorString(e));
    g_noalloc_small_ptr[dev] = q;
    g_noalloc_ptr[dev] = p;
  }
  *small = g_noalloc_small_ptr[dev];
  return g_noalloc_ptr[dev];
}

__constant__ Binom c_noalloc_binom;
bool g_noalloc_binom[kNoAllocMaxDevices] = {};

void noalloc_binomials(int dev, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_binom[dev]) {
    MB_CUDA(cudaMemcpyToSymbolAsync(c_noalloc_binom, &binom_table(), sizeof(Binom), 0,
                                    cudaMemcpyHostToDevice, st));
    MB_CUDA(cudaStreamSynchronize(st));
    g_noalloc_binom[dev] = true;
  }
}

// dst[i] = src[ref(i)] (GATHER) or dst[ref(i)] = src[i], with ref(i) the
// reference index of tensor state i computed on the fly.
template <typename V2, bool GATHER>
__global__ void k_noalloc_permute(OpView v, const V2* __restrict__ src, V2* __restrict__ dst) {
  __shared__ Binom sb;
  for (int i = threadIdx.x; i < (int)(sizeof(Binom) / sizeof(int64_t)); i += blockDim.x)
    (&sb.c[0][0])[i] = (&c_noalloc_binom.c[0][0])[i];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.dim;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ru = i / v.Dd, rd = i - ru * v.Dd;
    const int64_t ref = reference_rank(sb, v.up_mask[ru], v.dn_mask[rd], v.L);
    if (GATHER) dst[i] = src[ref];
    else dst[ref] = src[i];
  }
}

template <typename V2>
void noalloc_apply(mb_op_s* op, const void* x, void* y, int dev, cudaStream_t st) {
  void* small = nullptr;
  V2* a = reinterpret_cast<V2*>(noalloc_scratch(dev, &small));
  V2* b = a + kNoAllocMaxDim;
  const int grid = blas_grid(op->dim);
  k_noalloc_permute<V2, true><<<grid, 256, 0, st>>>(op->view, (const V2*)x, a);
  MB_CUDA(cudaGetLastError());
  launch_apply(op->view, op->precision, a, b, 1.0, 0.0, 0.0, nullptr, nullptr, 0, st);
  k_noalloc_permute<V2, false><<<grid, 256, 0, st>>>(op->view, b, (V2*)y);
  MB_CUDA(cudaGetLastError());
}

// MB_PREC_Q64: x permuted into a, converted to Q64 in b with the exponent
// of its largest element, the integer apply into a, converted back into b,
// permuted out -- the steps of mb_op_apply on a Q64 operator.
void noalloc_apply_q64(mb_op_s* op, const void* x, void* y, int dev, cudaStream_t st) {
  void* small = nullptr;
  double2* a = reinterpret_cast<double2*>(noalloc_scratch(dev, &small));
  double2* b = a + kNoAllocMaxDim;
  QParams* prm = reinterpret_cast<QParams*>(small);
  int* ints = reinterpret_cast<int*>(reinterpret_cast<char*>(small) + kNoAllocIntsAt);
  const int grid = blas_grid(op->dim);
  k_noalloc_permute<double2, true><<<grid, 256, 0, st>>>(op->view, (const double2*)x, a);
  MB_CUDA(cudaGetLastError());
  launch_f64_to_q(op->dim, a, nullptr, op->q_qbits, ints, b, st);
  launch_q_plan(q_plain_plan_input(op), ints + 1, prm, st);
  launch_apply_q(op->view, b, a, nullptr, prm, nullptr, nullptr, 0, st);
  launch_q_to_f64(op->dim, a, nullptr, &prm->ey, b, st);
  k_noalloc_permute<double2, false><<<grid, 256, 0, st>>>(op->view, b, (double2*)y);
  MB_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace mb

using namespace mb;

extern "C" int mb_op_apply_noalloc(mb_op_t op, const void* x_dev, void* y_dev, void* stream) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && y_dev, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(x_dev != y_dev, MB_ERR_INVALID_ARG, "x and y must not overlap");
    MB_REQUIRE(!op->natural_order && !op->view.n_blocks, MB_ERR_INVALID_ARG,
               "mb_op_apply_noalloc takes lattice operators of one (N_up, N_down) sector");
    MB_REQUIRE(op->dim <= kNoAllocMaxDim, MB_ERR_CAPACITY,
               "mb_op_apply_noalloc handles at most 1048576 basis states; this sector has " +
                   std::to_string(op->dim) + " (use mb_op_apply)");
    int dev = 0;
    MB_CUDA(cudaGetDevice(&dev));
    MB_REQUIRE(dev == op->device, MB_ERR_INVALID_ARG,
               "the operator's device must be the current device");
    MB_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, MB_ERR_CAPACITY,
               "mb_op_apply_noalloc supports device ordinals 0..63");
    cudaStream_t st = (cudaStream_t)stream;
    noalloc_binomials(dev, st);
    if (op->precision == MB_PREC_F32) noalloc_apply<float2>(op, x_dev, y_dev, dev, st);
    else if (op->precision == MB_PREC_Q64) noalloc_apply_q64(op, x_dev, y_dev, dev, st);
    else noalloc_apply<double2>(op, x_dev, y_dev, dev, st);
  });
}
