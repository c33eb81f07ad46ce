// rsg_energy.cuh -- launchers of the FP64 energy audit (rsg_energy.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pn {

template <typename R>
struct EnergyCells {
  const R *S[6];
  const double *comp;  // [rows][36] pseudo-inverse stiffness, row = material id
  const double *vol;   // [n] cell volumes, or null: vol_uniform for every cell
  double vol_uniform;
  int64_t n;
};

// blocks (= partial sums) a launch over n elements uses
int energy_blocks(int64_t n);

// part[b] = 1/2 sum of mass * |V|^2 over block b's share of the n nodes
cudaError_t launch_energy_nodes(int precision, const void *const V[3], const double *mass, int64_t n,
                                double *part, int nb, cudaStream_t st);

// part[b] = 1/2 sum of vol * S . comp[mat] S over block b's share of the n
// cells; mat is uint8 (grid form) or int32 (table form)
cudaError_t launch_energy_cells(int precision, const void *const S[6], const void *mat, bool mat_u8,
                                const double *comp, const double *vol, double vol_uniform, int64_t n,
                                double *part, int nb, cudaStream_t st);

}  // namespace pn
