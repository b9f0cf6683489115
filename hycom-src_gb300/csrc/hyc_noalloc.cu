// hyc_noalloc.cu -- advem on one slice with no device allocation.
//
// Some callers cannot allocate device memory when they call the advection:
// a model whose device memory is handed in full to its own pool allocator
// at start-up, or a time loop that must not call into the CUDA allocator
// (cudaMalloc/cudaFree can synchronise the whole device).  For them this
// file keeps the scratch the advem kernel needs -- the updated slice before
// it is copied into fld, and the per-cell land/sea byte mask -- in one
// file-scope __device__ array of fixed size.  Every GPU that loads the
// library holds this array until the process exits.
//
// Limits and sharing:
//   * at most kNoallocMaxCells = 2^21 cells per slice ((idm+2*nbdy) *
//     (jdm+2*nbdy)), i.e. 16 MiB of output slice plus 2 MiB of mask, and
//     nbdy <= 64; larger slices are rejected with HYC_ERR_ARG;
//   * the masks are checked as hyc_adv_init checks them: iu must be
//     ip(i)*ip(i-1) and iv ip(j)*ip(j-1) wherever the west / south neighbour
//     exists.  The check runs on the GPU beside the mask conversion and
//     sets a flag word in the scratch; the call reads the flag back before
//     it returns (so it returns after its GPU work) and answers
//     HYC_ERR_MASK if it is set;
//   * all calls on a device share the one array and it keeps the contents
//     of the last call.  The flag word must start at zero and is cleared
//     at the start of every call; nothing else has to: every call rewrites
//     the whole mask and writes every sea cell of the output slice before
//     reading it.  Calls whose GPU work overlaps (different streams or host
//     threads without ordering) race on the array; order them;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress with that device current) and caches it; make
//     that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <cstdio>
#include <mutex>

#include "../../include/hycom_adv.h"
#include "hyc_args.h"
#include "hyc_internal.h"

namespace {

constexpr long long kNoallocMaxCells = 1LL << 21;
constexpr int kNoallocMaxNbdy = 64;
constexpr long long kMaskOffsetBytes = kNoallocMaxCells * (long long)sizeof(double);
constexpr long long kFlagOffsetBytes = kMaskOffsetBytes + kNoallocMaxCells;  // one int: mask check
constexpr long long kScratchBytes = kFlagOffsetBytes + 256;

// The scratch.  In host code this name is a host-side stand-in, not a
// device address: only the address from cudaGetSymbolAddress may be
// passed to kernels.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDev = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDev] = {};

// ip/iu/iv (int32, one slice of ld1 x ld2) -> kernel mask byte
// ip | iu<<1 | iv<<2, and the bigrid consistency of iu/iv with ip (the
// check of hyc_adv_init): *bad is set where it fails
__global__ void noalloc_mask_kernel(const int32_t *ip, const int32_t *iu, const int32_t *iv, long long ld1,
                                    long long n, uint8_t *msk, int *bad) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const bool p = ip[t] != 0, u = iu[t] != 0, v = iv[t] != 0;
    const long long ia = t % ld1;
    if ((ia > 0 && u != (p && ip[t - 1] != 0)) || (t >= ld1 && v != (p && ip[t - ld1] != 0))) atomicOr(bad, 1);
    msk[t] = (uint8_t)((p ? hyc::kIP : 0) | (u ? hyc::kIU : 0) | (v ? hyc::kIV : 0));
  }
}

// errors are reported through hyc_last_error(NULL, ...)
int nerr(int code, const char *msg) {
  hyc::set_library_error(msg);
  return code;
}

}  // namespace

extern "C" int hyc_advem_noalloc(int32_t idm, int32_t jdm, int32_t nbdy, int32_t advtyp, double *fld,
                                 const double *fldc, const double *u, const double *v, const double *fco,
                                 const double *fcn, double posdef, const double *scal, const double *scali,
                                 double dt2, const int32_t *ip, const int32_t *iu, const int32_t *iv, void *stream) {
  if (idm < 1 || jdm < 1 || nbdy < 3 || nbdy > kNoallocMaxNbdy)
    return nerr(HYC_ERR_ARG, "hyc_advem_noalloc: bad sizes (need idm, jdm >= 1 and 3 <= nbdy <= 64)");
  if (!(advtyp == 0 || advtyp == 1 || advtyp == 2 || advtyp == 4))
    return nerr(HYC_ERR_ADVTYP, "hyc_advem_noalloc: advtyp must be 0, 1, 2 or 4");
  const int mbdy = advtyp == 0 ? 2 : 5;
  if (nbdy < mbdy) return nerr(HYC_ERR_NBDY, "hyc_advem_noalloc: nbdy < mbdy_advtyp(advtyp)");
  if (!fld || !u || !v || !fco || !fcn || !scal || !scali || !ip || !iu || !iv || (advtyp >= 2 && !fldc))
    return nerr(HYC_ERR_ARG, "hyc_advem_noalloc: null array");
  const long long ld1l = (long long)idm + 2LL * nbdy, ld2l = (long long)jdm + 2LL * nbdy;
  if (ld1l > kNoallocMaxCells || ld2l > kNoallocMaxCells || ld1l * ld2l > kNoallocMaxCells)
    return nerr(HYC_ERR_ARG, "hyc_advem_noalloc: slice larger than the 2^21-cell static scratch");
  const int ld1 = (int)ld1l, ld2 = (int)ld2l;
  const long long cells = ld1l * ld2l;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDev) return nerr(HYC_ERR_CUDA, "hyc_advem_noalloc: no CUDA device");
  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {  // once per device, with that device current
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return nerr(HYC_ERR_CUDA, "hyc_advem_noalloc: cudaGetSymbolAddress failed");
      g_scratch_addr[dev] = p;
    }
    base = g_scratch_addr[dev];
  }
  double *out = reinterpret_cast<double *>(base);
  uint8_t *msk = reinterpret_cast<uint8_t *>(base) + kMaskOffsetBytes;
  int *bad = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(base) + kFlagOffsetBytes);
  cudaStream_t s = (cudaStream_t)stream;

  if ((e = cudaMemsetAsync(bad, 0, sizeof(int), s)) != cudaSuccess) return nerr(HYC_ERR_CUDA, cudaGetErrorString(e));
  int bx = (int)((cells + 255) / 256);
  if (bx > 1024) bx = 1024;
  noalloc_mask_kernel<<<bx, 256, 0, s>>>(ip, iu, iv, ld1l, cells, msk, bad);
  if ((e = cudaGetLastError()) != cudaSuccess) return nerr(HYC_ERR_CUDA, cudaGetErrorString(e));

  hyc::TileArgs a;
  memset(&a, 0, sizeof a);
  const hyc::TileShape shape{32, 16};
  a.ii = idm;
  a.jj = jdm;
  a.nbdy = nbdy;
  a.ld1 = ld1;
  a.ld2 = ld2;
  a.slice = cells;
  a.ntx = (idm + shape.tx - 1) / shape.tx;
  a.nty = (jdm + shape.ty - 1) / shape.ty;
  a.mode = 1;
  a.msk = msk;
  a.scal = scal;
  a.scali = scali;
  a.uflx = u;
  a.vflx = v;
  a.fco = fco;
  a.fcn = fcn;
  a.dt2 = dt2;
  a.nfld = 1;
  a.f[0].nbase = fld;
  a.f[0].mbase = fldc ? fldc : fld;
  a.f[0].k_off = 0;
  a.f[0].kmin = 1;
  a.f[0].kmax = 1;
  a.f[0].posdef = posdef;
  a.out = out;
  a.kdm = 1;
  if ((e = hyc::launch_advect_tiles(advtyp, a, 1, shape, s)) != cudaSuccess)
    return nerr(HYC_ERR_CUDA, cudaGetErrorString(e));
  if ((e = hyc::launch_copy_back(a, 1, s)) != cudaSuccess) return nerr(HYC_ERR_CUDA, cudaGetErrorString(e));
  // the mask check: the copy back writes fld only where the masks are sea,
  // so with inconsistent masks fld holds a result the reference would not
  // give; the caller learns it here
  int flag = 0;
  if ((e = cudaMemcpyAsync(&flag, bad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return nerr(HYC_ERR_CUDA, cudaGetErrorString(e));
  if (flag) return nerr(HYC_ERR_MASK, "hyc_advem_noalloc: iu/iv inconsistent with ip (bigrid masks expected)");
  return HYC_OK;
}
