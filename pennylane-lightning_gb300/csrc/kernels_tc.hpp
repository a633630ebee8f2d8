// Tensor-core (tcgen05) application of dense 6-wire complex64 blocks
// (kernels_tc.cu).
#pragma once

#include "plgb_common.cuh"

namespace plgb {

// Tile geometry of a 6-wire block on an n-qubit register.  The tile's 12
// local bits (the block bits and the six lowest other bits) in ascending
// order give the local index jj.  Member index u (the block's own index,
// bit q = the q-th lowest block bit) and group index g (bit q = the q-th
// lowest other local bit) are bit permutations of jj.  The output stage in
// shared memory is XOR-swizzled on jj (a linear map of jj's bits 4-11 into
// bits 0-3) so that its writes per tensor-memory lane fall in distinct
// banks.
struct TcGeom {
    int lbit[12];
    int glob[64];
    int nglob;
    u64 ntiles;
    unsigned short jj_of_u[64];
    unsigned short jj_of_g[64];
    unsigned short hst[12];  // XOR mask of stage position per jj bit
    unsigned short st_of_u[64], st_of_g[64]; // swizzled stage positions of u and g alone
    unsigned short mat_of_u[64];             // row of the caller's matrix for member u
    // per-row parts of the kernel's thread maps (256 split and 256 epilogue
    // threads, 16 rows each): the full-index offsets of local index
    // jj_of_u[r << 2] (split row r) and of r << 8 (epilogue row r), and the
    // stage position of r << 8
    u64 split_row_off[16];
    u64 epi_row_off[16];
    unsigned short epi_row_st[16];
};

// false when the register is too small (fewer than 12 qubits) or the bits
// are not six distinct positions below n; bits6[0] = the matrix's most
// significant local bit (its first wire)
bool tc_geom_for(int n, const int *bits6, TcGeom &g);
// the shared-memory image of a row-major 64 x 64 complex64 matrix (first
// wire = most significant bit) for the geometry: its real form, rows and
// columns in member order, split into three BF16 parts (h, m, l) in the MMA
// operand layout
size_t tc_a_image_bytes();
void tc_build_a_image(const cx<float> *U, const TcGeom &geom, unsigned short *img);
// sv <- U on every group of the six bits (img: device copy of the image;
// err: device word set to 1 when a CTA gave up waiting for its MMAs)
void launch_dense6_tc(cudaStream_t s, cx<float> *sv, const TcGeom &geom, const unsigned short *a_img, int *err);

// whether complex64 dense 6-wire gates take the tensor-core kernel
bool tc_dense_enabled();
bool set_tc_dense_enabled(bool on);

} // namespace plgb
