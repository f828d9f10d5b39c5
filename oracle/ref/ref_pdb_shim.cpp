// Host entry point into the reference's own PDB reading path, for pinning qses_read_pdb.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py together with the reference's
// cpdb/cpdb.cpp (compiled where it lies in the checkout) into oracle/_ref/, which never
// enters version control.  It walks the parsed structure the way the QuickSES executable
// does (CudaSurf.cu:942-968) and returns coordinates and the element's first byte; the
// radius lookup is a 7-entry table the test applies.
#include <cstring>
#include "cpdb.h"

extern "C" {

// Returns the atom count; fills up to `cap` atoms.  -1 when the file cannot be parsed.
int ref_read_pdb(const char *path, float *xyz, char *element0, int cap) {
    pdb *P = initPDB();
    if (parsePDB((char *)path, P, (char *)"") != 0) {
        freePDB(P);
        return -1;
    }
    int n = 0;
    for (int c = 0; c < P->size; c++) {
        chain *C = &P->chains[c];
        for (atom *A = &C->residues[0].atoms[0]; A != NULL; A = A->next) {
            if (n < cap) {
                xyz[3 * n] = A->coor.x;
                xyz[3 * n + 1] = A->coor.y;
                xyz[3 * n + 2] = A->coor.z;
                element0[n] = A->element[0];
            }
            n++;
        }
    }
    freePDB(P);
    return n;
}

}  // extern "C"
