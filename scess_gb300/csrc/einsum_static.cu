// scess_einsum_static: the FP64 contraction of scess_einsum on caller-owned
// device buffers, for callers that cannot allocate device memory.
//
// Its only scratch (the offset tables of the contraction and the split-K
// partial sums) lives in one file-scope __device__ array of a fixed size.
// Host code never passes the array's name to a kernel: on the host that name is
// a stand-in, not a device address.  The device address is looked up with
// cudaGetSymbolAddress once per device and CUDA context, with that device
// current, and the looked-up pointer is what the kernels receive.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "scess_cc.h"

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB on every device using the library
constexpr int kMaxDevices = 64;
constexpr int kMaxRank = 6;

static __device__ __align__(256) unsigned char g_einsum_scratch[kScratchBytes];

std::mutex g_addr_mu;
void *g_addr[kMaxDevices];
unsigned long long g_addr_ctx[kMaxDevices];  // context id the address belongs to

// Unique id of the calling thread's current CUDA context (cuCtxGetId; ids are
// never reused within a process), 0 if the driver cannot tell.  After a
// cudaDeviceReset the device's next primary context has a new id, and the
// library's device code, with this array, is loaded into it anew.
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    cudaGetLastError();
  });
  CUcontext cx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&cx) == CUDA_SUCCESS && cx &&
      get_id(cx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of g_einsum_scratch on the current device, looked up once per
// device and context (again when the context has changed, e.g. after a
// cudaDeviceReset).
int scratch_address(int dev, void **out) {
  std::lock_guard<std::mutex> lock(g_addr_mu);
  const unsigned long long cid = current_context_id();
  if (!g_addr[dev] || cid == 0 || g_addr_ctx[dev] != cid) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_einsum_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      g_addr[dev] = nullptr;
      return SCESS_ERR_CUDA;
    }
    g_addr[dev] = p;
    g_addr_ctx[dev] = cid;
  }
  *out = g_addr[dev];
  return SCESS_OK;
}

// Whether p is memory of device dev that kernels can read and write (device or
// managed memory).  cudaPointerGetAttributes allocates nothing.
bool on_device(const void *p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

// Index group of the contraction (M: free labels of A, N: free labels of B,
// K: summed labels) with, per label, its extent and its strides in the two
// operands that carry it.
struct Group {
  int n = 0;
  int64_t ext[2 * kMaxRank];
  int64_t s0[2 * kMaxRank], s1[2 * kMaxRank];
};

struct TableDesc {
  Group g[3];        // M, N, K
  int64_t len[3];    // group sizes
  int64_t *out0[3];  // rowA, colB, kA
  int64_t *out1[3];  // rowC, colC, kB
};

// Offset tables from the label strides: element e of a group (labels in order,
// the first varying fastest) gets sum_l i_l * stride_l for each of its operands.
__global__ void fill_tables_kernel(TableDesc d) {
  const int64_t total = d.len[0] + d.len[1] + d.len[2];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int w = 0;
    int64_t r = e;
    while (r >= d.len[w]) r -= d.len[w++];
    const Group &g = d.g[w];
    const int64_t idx = r;
    int64_t o0 = 0, o1 = 0;
    for (int l = 0; l < g.n; l++) {
      const int64_t i = r % g.ext[l];
      r /= g.ext[l];
      o0 += i * g.s0[l];
      o1 += i * g.s1[l];
    }
    d.out0[w][idx] = o0;
    d.out1[w][idx] = o1;
  }
}

struct Operand {
  char lbl[kMaxRank];
  int nd = 0;
  int64_t ext[kMaxRank], str[kMaxRank];
  int find(char c) const {
    for (int i = 0; i < nd; i++)
      if (lbl[i] == c) return i;
    return -1;
  }
};

// Labels of one operand from spec[b, e) with its column-major strides.
bool operand(const char *spec, size_t b, size_t e, int32_t nd, const int64_t *ext, Operand &o) {
  if (nd < 1 || nd > kMaxRank || !ext || (int64_t)(e - b) != nd) return false;
  o.nd = nd;
  int64_t s = 1;
  for (int i = 0; i < nd; i++) {
    const char c = spec[b + i];
    if (!((c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'))) return false;
    for (int j = 0; j < i; j++)
      if (o.lbl[j] == c) return false;  // repeated label
    if (ext[i] <= 0) return false;
    o.lbl[i] = c;
    o.ext[i] = ext[i];
    o.str[i] = s;
    s *= ext[i];
  }
  return true;
}

bool add_label(Group &g, int64_t ext, int64_t s0, int64_t s1) {
  if (g.n >= 2 * kMaxRank) return false;
  g.ext[g.n] = ext;
  g.s0[g.n] = s0;
  g.s1[g.n] = s1;
  g.n++;
  return true;
}

}  // namespace

extern "C" int scess_einsum_static(const char *spec, double alpha, const double *A, int32_t a_nd,
                                   const int64_t *a_ext, const double *B, int32_t b_nd,
                                   const int64_t *b_ext, double beta, double *C, int32_t c_nd,
                                   const int64_t *c_ext, void *stream) {
  if (!spec || !A || !B || !C) return SCESS_ERR_INVALID;
  // spec "a,b->c" with every operand's labels
  const size_t len = std::strlen(spec);
  const char *comma = std::strchr(spec, ',');
  const char *arrow = std::strstr(spec, "->");
  if (!comma || !arrow || comma > arrow || len > 64) return SCESS_ERR_INVALID;
  Operand oa, ob, oc;
  const size_t ic = (size_t)(comma - spec), ia = (size_t)(arrow - spec);
  if (!operand(spec, 0, ic, a_nd, a_ext, oa) || !operand(spec, ic + 1, ia, b_nd, b_ext, ob) ||
      !operand(spec, ia + 2, len, c_nd, c_ext, oc))
    return SCESS_ERR_INVALID;

  // M / N: labels of C in C's order (from A / from B); K: labels of A absent from C
  TableDesc d;
  std::memset(&d, 0, sizeof(d));
  for (int i = 0; i < oc.nd; i++) {
    const char c = oc.lbl[i];
    const int pa = oa.find(c), pb = ob.find(c);
    if ((pa >= 0) == (pb >= 0)) return SCESS_ERR_INVALID;  // in neither or in both
    if (pa >= 0) {
      if (oa.ext[pa] != oc.ext[i] || !add_label(d.g[0], oc.ext[i], oa.str[pa], oc.str[i]))
        return SCESS_ERR_INVALID;
    } else {
      if (ob.ext[pb] != oc.ext[i] || !add_label(d.g[1], oc.ext[i], ob.str[pb], oc.str[i]))
        return SCESS_ERR_INVALID;
    }
  }
  for (int i = 0; i < oa.nd; i++) {
    const char c = oa.lbl[i];
    if (oc.find(c) >= 0) continue;
    const int pb = ob.find(c);
    if (pb < 0 || ob.ext[pb] != oa.ext[i] || !add_label(d.g[2], oa.ext[i], oa.str[i], ob.str[pb]))
      return SCESS_ERR_INVALID;
  }
  for (int i = 0; i < ob.nd; i++)
    if (oc.find(ob.lbl[i]) < 0 && oa.find(ob.lbl[i]) < 0) return SCESS_ERR_INVALID;

  // Each group has at most 6 labels of extent < 2^63 in total; cap the sizes
  // before multiplying them into the table length.
  int64_t M = 1, N = 1, K = 1;
  for (int w = 0; w < 3; w++) {
    int64_t p = 1;
    for (int l = 0; l < d.g[w].n; l++) {
      if (d.g[w].ext[l] > (int64_t(1) << 40) / p) return SCESS_ERR_TOO_LARGE;
      p *= d.g[w].ext[l];
    }
    (w == 0 ? M : w == 1 ? N : K) = p;
  }
  // scratch: rowA[M] kA[K] colB[N] kB[K] rowC[M] colC[N] (int64), then partials
  const int64_t table_bytes = 16 * (M + N + K);
  if (table_bytes > (int64_t)kScratchBytes) return SCESS_ERR_TOO_LARGE;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return SCESS_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return SCESS_ERR_UNSUPPORTED;
  // host memory, or another GPU's, would fault in the kernels: refuse it here
  if (!on_device(A, dev) || !on_device(B, dev) || !on_device(C, dev)) return SCESS_ERR_INVALID;
  void *base = nullptr;
  const int st = scratch_address(dev, &base);
  if (st != SCESS_OK) return st;

  int64_t *t = (int64_t *)base;
  int64_t *rowA = t, *kA = rowA + M, *colB = kA + K, *kB = colB + N, *rowC = kB + K,
          *colC = rowC + M;
  const int64_t part_off = scess::round_up(table_bytes, 256);
  double *partial = (double *)((unsigned char *)base + part_off);
  const int64_t part_doubles = ((int64_t)kScratchBytes - part_off) / 8;

  d.len[0] = M;
  d.len[1] = N;
  d.len[2] = K;
  d.out0[0] = rowA;
  d.out1[0] = rowC;
  d.out0[1] = colB;
  d.out1[1] = colC;
  d.out0[2] = kA;
  d.out1[2] = kB;

  scess::TableGemm g;
  g.A = A;
  g.B = B;
  g.C = C;
  g.rowA = rowA;
  g.kA = kA;
  g.colB = colB;
  g.kB = kB;
  g.rowC = rowC;
  g.colC = colC;
  g.M = M;
  g.N = N;
  g.K = K;
  g.alpha = alpha;
  g.beta = beta;
  g.aUnitM = d.g[0].n > 0 && d.g[0].s0[0] == 1;
  g.bUnitN = d.g[1].n > 0 && d.g[1].s0[0] == 1;

  const cudaStream_t s = (cudaStream_t)stream;
  try {
    const int64_t total = M + N + K;
    fill_tables_kernel<<<(unsigned)std::min<int64_t>(scess::ceil_div(total, 256), 4 * scess::kNumSMs),
                         256, 0, s>>>(d);
    SCESS_CHECK_LAUNCH();
    scess::dgemm_table_bounded(g, partial, part_doubles, s);
  } catch (const scess::Error &e) {
    return e.code;
  } catch (...) {
    return SCESS_ERR_CUDA;
  }
  return SCESS_OK;
}
