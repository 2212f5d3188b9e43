/* layout.h -- byte layouts of CabanaPIC's hot-path arrays.
 *
 * These are the reference's data layouts, kept unchanged so that buffers
 * allocated by a Kokkos/Cabana build of the reference can be passed to the
 * C-ABI as raw pointers (and vice versa):
 *
 *   particle_list_t      Cabana::AoSoA<MemberTypes<real_t x7, int>, MemorySpace>
 *                        (src/types.h:31-58).  SoA block s of vector length VL:
 *                          x[VL] y[VL] z[VL] ux[VL] uy[VL] uz[VL] w[VL] (real_t), cell[VL] (int)
 *                        Cabana's default VL is 32 on CUDA memory spaces, 16 on
 *                        host spaces; both are accepted.
 *   interpolator_array_t Cabana::AoSoA<real_t x18, MemorySpace, 32> (src/types.h:64-108)
 *   field_array_t        Cabana::AoSoA<real_t x9, MemorySpace, 32>  (src/types.h:138-172)
 *   accumulator_array_t  Kokkos::View<real_t*[3][4]> (src/types.h:116-134), taken in
 *                        LayoutRight: element (cell, comp, quadrant) at cell*12 + comp*4 + quadrant
 *
 * Cell indices are ghosted voxels: VOXEL(x,y,z) = x + (nx+2ng)*(y + (ny+2ng)*z)
 * (src/types.h:195).
 */
#ifndef CPIC_LAYOUT_H
#define CPIC_LAYOUT_H

#include <stddef.h>
#include <stdint.h>

#define CPIC_CELL_BLOCK 32          /* CELL_BLOCK_FACTOR, src/types.h:15-17 */
#define CPIC_INTERP_MEMBERS 18
#define CPIC_FIELD_MEMBERS 9
#define CPIC_ACC_VALUES 12          /* [3][4], src/types.h:116-120 */

/* particle members, src/types.h:31-41 */
enum cpic_particle_member {
  CPIC_PX = 0, CPIC_PY, CPIC_PZ, CPIC_UX, CPIC_UY, CPIC_UZ, CPIC_W, CPIC_CELL
};

/* interpolator members, src/types.h:64-84 */
enum cpic_interp_member {
  CPIC_I_EX = 0, CPIC_I_DEXDY, CPIC_I_DEXDZ, CPIC_I_D2EXDYDZ,
  CPIC_I_EY, CPIC_I_DEYDZ, CPIC_I_DEYDX, CPIC_I_D2EYDZDX,
  CPIC_I_EZ, CPIC_I_DEZDX, CPIC_I_DEZDY, CPIC_I_D2EZDXDY,
  CPIC_I_CBX, CPIC_I_DCBXDX, CPIC_I_CBY, CPIC_I_DCBYDY, CPIC_I_CBZ, CPIC_I_DCBZDZ
};

/* field members, src/types.h:138-149 */
enum cpic_field_member {
  CPIC_F_EX = 0, CPIC_F_EY, CPIC_F_EZ, CPIC_F_CBX, CPIC_F_CBY, CPIC_F_CBZ,
  CPIC_F_JFX, CPIC_F_JFY, CPIC_F_JFZ
};

/* bytes of one particle SoA block */
static inline size_t cpic_particle_block_bytes(int real_bytes, int vl) {
  return (size_t)vl * (size_t)(7 * real_bytes + 4);
}

/* bytes of an AoSoA particle list of n particles (whole SoA blocks) */
static inline size_t cpic_particle_list_bytes(int64_t n, int real_bytes, int vl) {
  return (size_t)((n + vl - 1) / vl) * cpic_particle_block_bytes(real_bytes, vl);
}

/* bytes of a cell AoSoA (interpolator: 18 members, field: 9 members) */
static inline size_t cpic_cell_array_bytes(int64_t num_cells, int members, int real_bytes) {
  return (size_t)((num_cells + CPIC_CELL_BLOCK - 1) / CPIC_CELL_BLOCK) * CPIC_CELL_BLOCK *
         (size_t)members * (size_t)real_bytes;
}

/* element offset (in real_t units) of member m of cell c in a cell AoSoA */
static inline size_t cpic_cell_offset(int64_t c, int members, int m) {
  return (size_t)(c / CPIC_CELL_BLOCK) * (size_t)(members * CPIC_CELL_BLOCK) +
         (size_t)m * CPIC_CELL_BLOCK + (size_t)(c % CPIC_CELL_BLOCK);
}

static inline int64_t cpic_voxel(int64_t x, int64_t y, int64_t z, int64_t nx, int64_t ny,
                                 int64_t ng) {
  return x + (nx + 2 * ng) * (y + (ny + 2 * ng) * z);
}

#endif /* CPIC_LAYOUT_H */
