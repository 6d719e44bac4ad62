/* hf_host_run - a C host driving the GB300 reacting-Euler step through the C ABI alone.
 *
 * The loop of BlockAMR::run (HyperFlow_V3/src/BlockAMR.cpp:400-423) for a uniform
 * single-patch level: create the stepper, load the state, take nsteps CFL Strang steps
 * (each with the reference's rollback and dt halving inside hf_stepper_step), read the
 * state back.  Plain C99, no CUDA headers: the state moves through host memory
 * (hf_stepper_set_host / hf_stepper_get_host).
 *
 *   hf_host_run CASE RESULT
 *
 * CASE (native byte order):
 *   char[8]   "HFCASE1"
 *   int32[12] nx, ny, periodic[2], bc_lo[2], bc_hi[2], nsteps, flux_form, chem_form, chemistry
 *   double[21] dx, dy, xlo, ylo, wedge_start, cfl, rtol, atol, inlet[13]
 *   char[32]  mechanism name ("H2_Li" or "H2_Li+AR")
 *   double[NV*ny*nx] initial state, SoA [NV][ny][nx]
 * RESULT:
 *   int32     steps taken
 *   double    final time
 *   double[nsteps] accepted step sizes
 *   double[NV*ny*nx] final state, SoA [NV][ny][nx]
 * Exit status: 0 on success, 1 on a solver error (message on stderr), 2 on bad usage or I/O.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hyperflow_gpu.h"

static int fail_io(const char* what, const char* path) {
    fprintf(stderr, "hf_host_run: cannot %s %s\n", what, path);
    return 2;
}

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: hf_host_run CASE RESULT\n"
                        "  CASE: level, steps and initial state (see the source header); RESULT: steps,\n"
                        "  time, step sizes and final state\n");
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return fail_io("open", argv[1]);
    char magic[8];
    int32_t iv[12];
    double dv[21];
    char mech[33];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "HFCASE1", 7) != 0 || fread(iv, sizeof(int32_t), 12, f) != 12 ||
        fread(dv, sizeof(double), 21, f) != 21 || fread(mech, 1, 32, f) != 32) {
        fclose(f);
        return fail_io("read the header of", argv[1]);
    }
    mech[32] = '\0';
    const int nx = iv[0], ny = iv[1], nsteps = iv[8];
    if (nx <= 0 || ny <= 0 || nsteps < 0) {
        fclose(f);
        return fail_io("use the level of", argv[1]);
    }

    hf_ctx* ctx = NULL;
    if (hf_init(mech, 0, &ctx) != HF_OK) {
        fclose(f);
        fprintf(stderr, "hf_host_run: hf_init(%s) failed\n", mech);
        return 1;
    }
    const int nv = hf_nspecies(ctx) + 3;
    const size_t ncell = (size_t)nx * (size_t)ny;
    double* state = (double*)malloc(sizeof(double) * (size_t)nv * ncell);
    double* dts = (double*)calloc((size_t)(nsteps > 0 ? nsteps : 1), sizeof(double));
    if (!state || !dts || fread(state, sizeof(double), (size_t)nv * ncell, f) != (size_t)nv * ncell) {
        fclose(f);
        free(state);
        free(dts);
        hf_destroy(ctx);
        return fail_io("read the state of", argv[1]);
    }
    fclose(f);

    hf_level L;
    memset(&L, 0, sizeof L);
    L.nx = nx;
    L.ny = ny;
    L.periodic[0] = iv[2];
    L.periodic[1] = iv[3];
    L.bc_lo[0] = iv[4];
    L.bc_lo[1] = iv[5];
    L.bc_hi[0] = iv[6];
    L.bc_hi[1] = iv[7];
    L.dx = dv[0];
    L.dy = dv[1];
    L.xlo = dv[2];
    L.ylo = dv[3];
    L.wedge_start = dv[4];
    for (int n = 0; n < 13; ++n) L.inlet[n] = dv[8 + n];
    const double cfl = dv[5], rtol = dv[6], atol = dv[7];

    int rc = 0, taken = 0;
    hf_stepper* st = NULL;
    hf_status r = hf_stepper_create(ctx, &L, NULL, iv[11], rtol, atol, iv[9], iv[10], &st);
    if (r == HF_OK) r = hf_stepper_set_host(st, state, NULL);
    for (; r == HF_OK && taken < nsteps; ++taken) {
        double dt = 0.0; /* <= 0: the CFL step (stableDt) */
        r = hf_stepper_step(st, cfl, &dt, NULL);
        if (r == HF_OK) dts[taken] = dt;
    }
    if (r == HF_OK) r = hf_stepper_get_host(st, state, NULL);
    if (r != HF_OK) {
        fprintf(stderr, "hf_host_run: step %d failed (status %d): %s\n", taken, (int)r, hf_last_error(ctx));
        rc = 1;
    } else {
        FILE* o = fopen(argv[2], "wb");
        const int32_t t32 = taken;
        const double time = hf_stepper_time(st);
        if (!o || fwrite(&t32, sizeof t32, 1, o) != 1 || fwrite(&time, sizeof time, 1, o) != 1 ||
            fwrite(dts, sizeof(double), (size_t)nsteps, o) != (size_t)nsteps ||
            fwrite(state, sizeof(double), (size_t)nv * ncell, o) != (size_t)nv * ncell)
            rc = fail_io("write", argv[2]);
        if (o) fclose(o);
    }
    if (st) hf_stepper_destroy(st);
    hf_destroy(ctx);
    free(state);
    free(dts);
    return rc;
}
