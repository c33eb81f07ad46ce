// rsg_grid_tma.cu -- the tensor-copy grid step (rsg_grid_tma.cuh) with 32 x 8
// tiles for every storage type, the tensor-map encoding, and the launch
// dispatch (32 x 16 FP32 tiles come from rsg_grid_tma16.cu, the FP64 form's
// per-block path kernels from rsg_grid_tma_f64.cu).
#include "rsg_grid_tma.cuh"

namespace pn {

// rsg_grid_tma16.cu
cudaError_t launch_grid_tma_f32_rows16(const GridArgs<float> &a, int sym, cudaStream_t st);
cudaError_t launch_grid_tma_batch_f32_rows16(const GridBatchLaunch &b, int step, cudaStream_t st);
int grid_tma_blocks_per_sm_f32_rows16();
// rsg_grid_tma_f64.cu
cudaError_t launch_grid_tma_f64h(const GridArgs<double> &a, int sym, cudaStream_t st);
cudaError_t launch_grid_tma_batch_f64h(const GridBatchLaunch &b, int step, cudaStream_t st);

namespace {

// ---- tensor-map encoding (driver entry point, no libcuda link) ------------------
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                 CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                 CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static const EncodeTiled fn = []() -> EncodeTiled {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// L2 sector promotion of the tile copies (tuning override PN_TMA_L2_PROMOTION
// = 0, 64, 128 or 256 bytes; default 128)
CUtensorMapL2promotion l2_promotion() {
  const char *v = std::getenv("PN_TMA_L2_PROMOTION");
  const int b = v ? std::atoi(v) : 128;
  return b == 0 ? CU_TENSOR_MAP_L2_PROMOTION_NONE
       : b == 64 ? CU_TENSOR_MAP_L2_PROMOTION_L2_64B
       : b == 256 ? CU_TENSOR_MAP_L2_PROMOTION_L2_256B
                  : CU_TENSOR_MAP_L2_PROMOTION_L2_128B;
}

// 3-D tile map over a pitched lattice buffer: dims (d0, d1, d2) sites, rows of
// `pitch` sites, box (b0, b1, 1)
bool encode3(CUtensorMap *m, CUtensorMapDataType dt, int esz, const void *ptr, int64_t d0, int64_t d1,
             int64_t d2, int64_t pitch, int b0, int b1) {
  const EncodeTiled fn = encoder();
  if (!fn || !ptr) return false;
  if (((uintptr_t)ptr & 15) != 0 || (pitch * esz) % 16 != 0 || (b0 * esz) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
  const cuuint64_t strides[2] = {(cuuint64_t)(pitch * esz), (cuuint64_t)(pitch * d1 * esz)};
  const cuuint32_t box[3] = {(cuuint32_t)b0, (cuuint32_t)b1, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, dt, 3, const_cast<void *>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, l2_promotion(), CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// boxes of a 32 x ty tile: stress (ty + 1 rows with the -y apron row), node
// fields (ty rows), material bytes (ty - 1 rows, the owned cells)
template <int ESZ>
bool encode_all(int ty, int nx, int ny, int nz, int pnx, int pcx, const void *const V[3], const void *const S[6],
                const void *coef, const uint8_t *mat, GridMaps &m) {
  using G = Geo<ESZ, 8>;  // box widths do not depend on the rows
  const CUtensorMapDataType dt = ESZ == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT64;
  bool ok = true;
  for (int f = 0; f < 6; f++) ok = ok && encode3(&m.S[f], dt, ESZ, S[f], nx, ny, nz, pcx, G::BWC, ty + 1);
  for (int c = 0; c < 3; c++) ok = ok && encode3(&m.V[c], dt, ESZ, V[c], nx + 1, ny + 1, nz + 1, pnx, G::BWN, ty);
  ok = ok && encode3(&m.coef, dt, ESZ, coef, nx + 1, ny + 1, nz + 1, pnx, G::BWN, ty);
  ok = ok && encode3(&m.mat, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, mat, nx, ny, nz, pcx, G::BWM, ty - 1);
  return ok;
}

}  // namespace

size_t grid_tma_maps_bytes() { return sizeof(GridMaps); }

bool grid_tma_rows_supported(int precision, int tile_rows) {
  return tile_rows == 8 || (tile_rows == 16 && precision == 2);
}

bool grid_tma_encode(int precision, int tile_rows, int nx, int ny, int nz, int pnx, int pcx,
                     const void *const V[3], const void *const S[6], const void *coef, const uint8_t *mat,
                     void *out) {
  if (!grid_tma_rows_supported(precision, tile_rows)) return false;
  GridMaps m;
  std::memset(&m, 0, sizeof(m));
  const bool ok = precision == 2 ? encode_all<4>(tile_rows, nx, ny, nz, pnx, pcx, V, S, coef, mat, m)
                                 : encode_all<8>(tile_rows, nx, ny, nz, pnx, pcx, V, S, coef, mat, m);
  if (ok) std::memcpy(out, &m, sizeof(m));
  return ok;
}

int grid_tma_blocks_per_sm(int precision, int tile_rows) {
  if (!grid_tma_rows_supported(precision, tile_rows)) return 0;
  if (tile_rows == 16) return grid_tma_blocks_per_sm_f32_rows16();
  int sms = 0, per_sm = 0;
  const cudaError_t e = precision == 2 ? SetupT<float, 0, 8>::ensure(sms, per_sm)
                      : precision == 3 ? SetupT<df64, 0, 8>::ensure(sms, per_sm)
                                       : SetupT<double, 0, 8>::ensure(sms, per_sm);
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_grid_tma(const void *args, int precision, int sym, cudaStream_t st) {
  if (precision == 2) {
    const GridArgs<float> &a = *(const GridArgs<float> *)args;
    if (a.tile_rows == 16) return launch_grid_tma_f32_rows16(a, sym, st);
    if (a.tile_rows != 8) return cudaErrorInvalidValue;
    return launch_sym<float, 8>(a, sym, st);
  }
  if (precision == 3) {
    const GridArgs<float2> &a = *(const GridArgs<float2> *)args;
    if (a.tile_rows != 8) return cudaErrorInvalidValue;
    return launch_sym<df64, 8>(a, sym, st);
  }
  const GridArgs<double> &a = *(const GridArgs<double> *)args;
  if (a.tile_rows != 8) return cudaErrorInvalidValue;
  if (a.rflags) return launch_grid_tma_f64h(a, sym, st);  // the FP64 form: per-block double-float / FP64 path
  return launch_sym<double, 8>(a, sym, st);
}

cudaError_t launch_grid_tma_batch(const GridBatchLaunch &b, int precision, int step, cudaStream_t st) {
  if (!grid_tma_rows_supported(precision, b.tile_rows)) return cudaErrorInvalidValue;
  if (precision == 2)
    return b.tile_rows == 16 ? launch_grid_tma_batch_f32_rows16(b, step, st) : launch_batch_sym<float, 8>(b, step, st);
  if (precision == 3) return launch_batch_sym<df64, 8>(b, step, st);
  if (b.range_flags) return launch_grid_tma_batch_f64h(b, step, st);
  return launch_batch_sym<double, 8>(b, step, st);
}

}  // namespace pn
