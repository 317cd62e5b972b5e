// pn_noalloc.cu -- a force evaluation that allocates nothing.
//
// Some callers of this library cannot allocate GPU memory when they need a force: a host
// framework that owns all device memory through its own pool (a raw cudaMalloc would bypass
// its accounting or fail against its reservation), a time-critical loop in which cudaMalloc /
// cudaFree would stall (they can synchronize the device), or a plug-in host that forbids
// allocations after start-up.  pn_force_noalloc serves them: the caller passes the inputs and
// the output buffer, and every work buffer of the evaluation (BH-relative positions, j-pack,
// tile origins, pair sums, reduction partials, counters) lives in one file-scope device array of
// PN_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the library holds that array until the
// process exits.
//
// The array's host-side name is only a stand-in for the symbol; its device address is obtained
// once per device, with that device current, by cudaGetSymbolAddress (checked) on the first
// call made on that device -- so that first call must come before any stream capture.
// Calls share the array and it keeps the last call's contents: the reduction counters and the
// error word are cleared at the start of every call (cudaMemsetAsync on the caller's stream),
// everything else is written before it is read.  Calls whose executions overlap on the GPU (on
// different streams, or on one device from several host threads) race on the array.
//
// Device-side outcomes (a non-finite force, e.g. a star exactly on the BH; an in-kernel wait
// that gave up) are recorded in the array's error word; pn_noalloc_status() waits for the
// caller's stream and reads that word into a host variable (a plain device-to-host copy, no
// allocation), so the caller learns them without allocating anything either.
//
// The per-device set-up (symbol address, SM count) is published through atomics: two host
// threads making their first call on one device at the same time both look the values up and
// store the same result, which is well defined.
#include <atomic>
#include <cstdio>

#include "../../include/pn.h"
#include "pn_kernels.h"

using namespace pn;

namespace {

constexpr int kMaxN = PN_NOALLOC_NMAX;           // particles, BH included
constexpr int kNpad = ((kMaxN - 1 + 255) / 256) * 256;
constexpr int kMaxSplits = 4;                     // j-range splits of the pair sweep
constexpr int kBlocks = kNpad / 256 + 2;

// byte offsets of the work buffers inside the array (each 256-byte aligned)
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffSpos = 0;
constexpr size_t kOffPack = kOffSpos + align256(3 * (size_t)kNpad * 8);
constexpr size_t kOffTorg = kOffPack + align256(6 * (size_t)kNpad * 16);
constexpr size_t kOffAcc = kOffTorg + align256(((size_t)kNpad / 32 + 1) * sizeof(TileOrigin));
constexpr size_t kOffPart = kOffAcc + align256((size_t)kMaxSplits * NACC_MAX * kNpad * 8);
constexpr size_t kOffGlob = kOffPart + align256((size_t)kBlocks * 8 * 2 * 8);
constexpr size_t kOffTick = kOffGlob + align256(16 * 8);
constexpr size_t kOffErr = kOffTick + 256;
constexpr size_t kBytes = kOffErr + 256;
static_assert(kBytes == PN_NOALLOC_SCRATCH_BYTES, "PN_NOALLOC_SCRATCH_BYTES must match the layout");

}  // namespace

// The scratch array itself (device memory, zero at load).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

namespace {
constexpr int kMaxDevices = 64;
// per device: the device address of g_noalloc_scratch and the SM count (0 = not looked up yet)
std::atomic<unsigned char *> g_dev_ptr[kMaxDevices];
std::atomic<int> g_dev_sms[kMaxDevices];
thread_local int g_noalloc_err = PN_OK;
}  // namespace

// Device address of the scratch array and the SM count of the current device (looked up on
// the first call made on that device, with that device current).
static int scratch_address(unsigned char **out, int *sms_out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return PN_ERR_UNSUPPORTED;
    }
    unsigned char *ptr = g_dev_ptr[dev].load(std::memory_order_acquire);
    int sms = g_dev_sms[dev].load(std::memory_order_acquire);
    if (!ptr || sms <= 0) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "libpn: cudaGetSymbolAddress(scratch) failed: %s\n", cudaGetErrorString(e));
            cudaGetLastError();
            return PN_ERR_CUDA;
        }
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            return PN_ERR_CUDA;
        }
        ptr = static_cast<unsigned char *>(p);
        g_dev_sms[dev].store(sms, std::memory_order_release);
        g_dev_ptr[dev].store(ptr, std::memory_order_release);
    }
    *out = ptr;
    if (sms_out) *sms_out = sms;
    return PN_OK;
}

extern "C" int pn_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int pn_noalloc_status(void *stream) {
    unsigned char *base = nullptr;
    int rc = scratch_address(&base, nullptr);
    if (rc) return rc;
    if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess) {
        cudaGetLastError();
        return PN_ERR_CUDA;
    }
    int word = 0;  // a host stack variable: the copy allocates nothing
    if (cudaMemcpy(&word, base + kOffErr, sizeof word, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return PN_ERR_CUDA;
    }
    if (word & DEVERR_TIMEOUT) return PN_ERR_TIMEOUT;
    if (word & DEVERR_NONFINITE) return PN_ERR_NONFINITE;
    return PN_OK;
}

extern "C" int pn_force_noalloc(int n, const double *d_x, const double *d_v, const double *d_m,
                                double eps, double inv_c2, int precision, double *d_a, void *stream) {
    auto fail = [](int code) {
        g_noalloc_err = code;
        return code;
    };
    if (n < 1 || n > kMaxN) {
        fprintf(stderr, "libpn: pn_force_noalloc: n = %d outside [1, %d] (PN_NOALLOC_NMAX)\n", n, kMaxN);
        return fail(PN_ERR_INVALID);
    }
    if (!d_x || !d_v || !d_m || !d_a || !(eps > 0.0) || !(inv_c2 >= 0.0) ||
        (precision != PN_PREC_FP64 && precision != PN_PREC_MIXED))
        return fail(PN_ERR_INVALID);
    unsigned char *base = nullptr;
    int sms = 0;
    int rc = scratch_address(&base, &sms);
    if (rc) return fail(rc);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *spos = reinterpret_cast<double *>(base + kOffSpos);
    void *pack = base + kOffPack;
    TileOrigin *torg = reinterpret_cast<TileOrigin *>(base + kOffTorg);
    double *acc = reinterpret_cast<double *>(base + kOffAcc);
    double *part = reinterpret_cast<double *>(base + kOffPart);
    double *glob = reinterpret_cast<double *>(base + kOffGlob);
    unsigned *tickets = reinterpret_cast<unsigned *>(base + kOffTick);
    int *err = reinterpret_cast<int *>(base + kOffErr);
    if (cudaMemsetAsync(base + kOffTick, 0, 512, s) != cudaSuccess) {  // counters + error word
        cudaGetLastError();
        return fail(PN_ERR_CUDA);
    }

    const int nstar = n - 1;
    const bool f32 = precision == PN_PREC_MIXED;
    const int mode = inv_c2 != 0.0 ? MODE_FORCE : MODE_NEWTON;
    PairCfg k;
    k.ipt = f32 ? 2 : 1;
    k.js = 1;
    k.tj = f32 ? 128 : 64;
    const int bi = PAIR_NT * k.ipt;
    const int nib = (nstar + bi - 1) / bi;
    const int ntiles = (nstar + k.tj - 1) / k.tj;
    int g = nib > 0 ? (4 * sms * 4 + nib - 1) / nib : 1;  // about 4 waves of 4 CTAs per SM
    if (g > kMaxSplits) g = kMaxSplits;
    if (g > ntiles) g = ntiles;
    if (g < 1) g = 1;
    k.gsplit = g;
    const double eps2 = eps * eps;

    PrepArgs pa{};
    pa.x = d_x; pa.v = d_v; pa.m = d_m; pa.sp = 3; pa.sk = 1;
    pa.nstar = nstar; pa.npad = kNpad; pa.nfill = ((nstar > 0 ? nstar : 1) + 255) / 256 * 256;
    pa.tj = k.tj; pa.f32 = f32; pa.eps2 = eps2;
    pa.pack = pack; pa.torg = torg; pa.spos = spos; pa.part = part; pa.glob = glob;
    pa.ticket = &tickets[0];
    if (launch_prep(pa, s) != cudaSuccess) return fail(PN_ERR_CUDA);
    if (nstar > 0) {
        PairArgs qa{};
        qa.pack = pack; qa.torg = torg; qa.spos = spos; qa.out = acc; qa.err = err;
        qa.nstar = nstar; qa.npad = kNpad; qa.tj = k.tj; qa.ntiles = ntiles; qa.gsplit = k.gsplit;
        qa.eps2 = eps2;
        const cudaError_t e = f32 ? launch_pair_f32(mode, k, qa, s) : launch_pair_f64(mode, k, qa, s);
        if (e != cudaSuccess) return fail(PN_ERR_CUDA);
    }
    FinishArgs fa{};
    fa.v = d_v; fa.m = d_m; fa.vsp = 3; fa.vsk = 1;
    fa.spos = spos; fa.acc = acc; fa.glob = glob;
    fa.nstar = nstar; fa.npad = kNpad; fa.nacc = pair_nacc(mode); fa.gsplit = k.gsplit;
    fa.pn1 = mode == MODE_FORCE;
    fa.eps = eps; fa.eps2 = eps2; fa.inv_c2 = inv_c2; fa.dt = 0.0;
    fa.a = d_a; fa.asp = 3; fa.ask = 1; fa.stage = 0;
    fa.part = part + (size_t)kBlocks * 8;
    fa.ticket = &tickets[1]; fa.err = err;
    if (launch_finish(fa, s) != cudaSuccess) return fail(PN_ERR_CUDA);
    return fail(PN_OK);
}
