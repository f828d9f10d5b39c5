// QuickSES-compatible command line (CudaSurf.cu:875-975):
//   QuickSES -i input.pdb -o output.obj [-l passes=1] [-v voxel=0.5] [-s slice=300] [-h]
// -i and -o are mandatory; a missing one prints the usage and exits with -1, like the
// reference's argument validation.  Degenerate triangles are kept, as the reference's OBJ
// path keeps them.  By default the mesh is the reference's single-slice result whatever -s
// is; with -r it is the reference's sliced output for slices of -s voxels (each slice
// meshed, welded and smoothed on its own, the OBJ holding the slices one after the other,
// CudaSurf.cu:329-371, 629-754).
// Extra: -r (the reference's slicing), -d device (default 0), -t (stage times to stderr).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "quickses.h"

namespace {

void usage(const char *prog) {
    fprintf(stderr,
            "  %s {OPTIONS}\n\n"
            "    QuickSES, SES mesh generation using GPU\n\n"
            "  OPTIONS:\n\n"
            "      -i[input.pdb]                     Input PDB file\n"
            "      -o[output.obj]                    Output OBJ mesh file\n"
            "      -l[smooth factor]                 (1) Times to run Laplacian smoothing step.\n"
            "      -v[voxel size]                    (0.5) Voxel size in Angstrom. Defines the quality of the mesh.\n"
            "      -s[slice size]                    (300) Size of the sub-grid (used with -r).\n"
            "      -r                                The reference's slicing: one mesh per sub-grid of -s\n"
            "                                        voxels, as QuickSES writes it.\n"
            "      -d[device]                        (0) CUDA device.\n"
            "      -t                                Print per-stage device times.\n"
            "      -h, --help                        Display this help menu\n",
            prog);
}

// Value of a flag given as "-x value" or "-xvalue".
bool take_value(int argc, const char **argv, int &k, std::string &out) {
    const char *a = argv[k];
    if (a[2]) {
        out = a + 2;
        return true;
    }
    if (k + 1 >= argc) return false;
    out = argv[++k];
    return true;
}

bool parse_int(const std::string &s, int &v) {
    char *end = nullptr;
    long x = strtol(s.c_str(), &end, 10);
    if (s.empty() || *end) return false;
    v = (int)x;
    return true;
}

bool parse_float(const std::string &s, float &v) {
    char *end = nullptr;
    float x = strtof(s.c_str(), &end);
    if (s.empty() || *end) return false;
    v = x;
    return true;
}

}  // namespace

int main(int argc, const char **argv) {
    std::string in, out;
    int passes = 1, slice = 300, device = 0;
    float voxel = 0.5f;
    bool times = false, slices = false;
    for (int k = 1; k < argc; k++) {
        const char *a = argv[k];
        if (!strcmp(a, "-h") || !strcmp(a, "--help")) {
            usage(argv[0]);
            return 0;
        }
        if (a[0] != '-' || !a[1]) {
            fprintf(stderr, "Passed in argument, but no positional arguments were ready to receive it: %s\n", a);
            usage(argv[0]);
            return -1;
        }
        std::string val;
        const char f = a[1];
        if (f == 't' && !a[2]) {
            times = true;
            continue;
        }
        if (f == 'r' && !a[2]) {
            slices = true;
            continue;
        }
        if (!strchr("iolvsd", f) || !take_value(argc, argv, k, val)) {
            fprintf(stderr, "Flag could not be matched or is missing its argument: %s\n", a);
            usage(argv[0]);
            return -1;
        }
        bool ok = true;
        switch (f) {
            case 'i': in = val; break;
            case 'o': out = val; break;
            case 'l': ok = parse_int(val, passes); break;
            case 'v': ok = parse_float(val, voxel); break;
            case 's': ok = parse_int(val, slice); break;
            case 'd': ok = parse_int(val, device); break;
        }
        if (!ok) {
            fprintf(stderr, "Argument '%s' received invalid value type '%s'\n", a, val.c_str());
            usage(argv[0]);
            return -1;
        }
    }
    if (in.empty() || out.empty()) {
        fprintf(stderr, "Usage: ");
        usage(argv[0]);
        return -1;
    }
    if (slices && slice < 1) {  // the reference would loop forever (CudaSurf.cu:653)
        fprintf(stderr, "Argument '-s' must be at least 1 with -r\n");
        return -1;
    }

    float *xyz = nullptr, *rad = nullptr;
    unsigned n = 0;
    if (qses_read_pdb(in.c_str(), &xyz, &rad, &n) != QSES_OK) {
        perror("pdb file can not read");
        return 2;
    }
    fprintf(stderr, "Grid resolution = %g\n", voxel);

    qses_context *ctx = nullptr;
    int rc = qses_context_create(device, nullptr, &ctx);
    if (rc != QSES_OK) {
        fprintf(stderr, "QuickSES: %s\n", qses_status_string(rc));
        return 1;
    }
    qses_set_profiling(ctx, times ? 1 : 0);
    qses_params p;
    qses_params_default(&p);
    p.voxel = voxel;
    p.smooth_passes = passes < 0 ? 0 : passes;
    p.slice = slice;
    p.flags = QSES_FLAG_KEEP_DEGENERATE | (slices ? QSES_FLAG_REFERENCE_SLICES : 0);
    qses_mesh m;
    rc = qses_compute(ctx, &p, (const qses_float3 *)xyz, rad, n, &m);
    if (rc != QSES_OK) {
        fprintf(stderr, "QuickSES: %s\n", qses_last_error(ctx));
        qses_context_destroy(ctx);
        return 1;
    }
    if (times) {
        float ms[32];
        const char *names[32];
        const int k = qses_stage_times(ctx, ms, names, 32);
        for (int q = 0; q < k; q++) fprintf(stderr, "  %-14s %8.3f ms\n", names[q], ms[q]);
    }
    fprintf(stderr, "%u atoms -> %u vertices, %u triangles\n", n, m.n_vertices, m.n_triangles);
    rc = qses_write_obj(out.c_str(), m.vertices, m.n_vertices, m.triangles, m.n_triangles, 0);
    if (rc != QSES_OK) fprintf(stderr, "Failed to open output file\n");
    qses_mesh_release(&m);
    qses_context_destroy(ctx);
    qses_free(xyz);
    qses_free(rad);
    return rc == QSES_OK ? 0 : -1;
}
