// Neighbour-cell key per atom (hashAtoms + spaceToGrid + flatten3DTo1D, Kernels.cu:119-131,
// 185-216).
//
// This translation unit is compiled with -use_fast_math, like the reference, and spells the
// cell coordinate as the same expression (p - o) / cell truncated to int, so the compiler
// emits the same approximate division.  That matters: the grid origin is min - maxR - probe,
// which puts the atom with the smallest coordinate of each axis exactly on a cell boundary,
// where the approximate quotient (just below the integer) and the IEEE one (exactly the
// integer) pick different cells.  The cell key only orders the atoms (the sorted order
// behind API_getAtomIdPerVert); which atoms the field sees does not depend on it.
#include "kernels.h"

namespace qses {

__global__ void k_atom_hash(QGrid g, const float *__restrict__ xyz, unsigned n, unsigned *__restrict__ key) {
    unsigned a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int cx = (int)((xyz[3 * a] - g.ox) / g.cell);
    const int cy = (int)((xyz[3 * a + 1] - g.oy) / g.cell);
    const int cz = (int)((xyz[3 * a + 2] - g.oz) / g.cell);
    key[a] = (unsigned)(g.gnb * g.gnb * cx + g.gnb * cy + cz);
}

// Batch form: the key of an atom of molecule m is offset by m's first cell, so one stable
// sort orders every molecule's atoms exactly as its own sort would, molecule after molecule.
__global__ void k_atom_hash_batch(QBatch b, const float *__restrict__ xyz, unsigned n, unsigned *__restrict__ key) {
    unsigned a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const unsigned m = qses_find(b.atom_off, b.n_mol, a);
    const QGrid g = b.mols[m].g;
    const int cx = (int)((xyz[3 * a] - g.ox) / g.cell);
    const int cy = (int)((xyz[3 * a + 1] - g.oy) / g.cell);
    const int cz = (int)((xyz[3 * a + 2] - g.oz) / g.cell);
    key[a] = b.mols[m].cell_off + (unsigned)(g.gnb * g.gnb * cx + g.gnb * cy + cz);
}

void launch_atom_hash(const QGrid &g, const float *xyz, unsigned n, unsigned *key, cudaStream_t s) {
    k_atom_hash<<<(n + 255) / 256, 256, 0, s>>>(g, xyz, n, key);
}
void launch_atom_hash_batch(const QBatch &b, const float *xyz, unsigned n, unsigned *key, cudaStream_t s) {
    k_atom_hash_batch<<<(n + 255) / 256, 256, 0, s>>>(b, xyz, n, key);
}

}  // namespace qses
