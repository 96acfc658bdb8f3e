/* A plain C99 caller of include/mcg.h: the calls a C or Fortran-side integration makes, in the
 * order the library's integration notes give them.  Built by tests/test_c_api.py with
 * -std=c99 -Wall -Wextra -Werror -pedantic and linked against libmcgpu.so.
 *
 * usage: host_calls SYSTEM.cor SYSTEM.ff
 * Without a device it runs the host-side calls (MDBAS reader, exclusion and 1-4 lists) and checks
 * that the device calls fail with MCG_ECUDA; with a device it also computes one energy and one
 * dE.  Prints "key value" lines. */
#include <stdio.h>
#include <stdlib.h>

#include "mcg.h"

static int report(const char* what, int rc) {
    printf("%s %d\n", what, rc);
    if (rc != MCG_OK) printf("%s_error %s\n", what, mcg_last_error()[0] ? "set" : "empty");
    return rc;
}

int main(int argc, char** argv) {
    mcg_mdbas* m = NULL;
    mcg_system_desc d = {0};
    mcg_system* s = NULL;
    mcg_batch* b = NULL;
    mcg_batch_opts o = {0};
    int* counts;
    int64_t total = 0;
    int n14 = 0, rc;
    double ener[10];

    if (argc != 3) return 2;
    printf("abi %d\n", mcg_abi_version());
    printf("devices %d\n", mcg_device_count());
    if (report("mdbas_read", mcg_mdbas_read(argv[1], argv[2], &m)) != MCG_OK) return 3;
    report("mdbas_fill", mcg_mdbas_fill(m, &d));
    printf("natom %d\n", mcg_mdbas_natom(m));
    d.pbc_type = MCG_PBC_CUBIC;
    d.box[0] = d.box[1] = d.box[2] = 24.6;
    d.cut_mode = MCG_CUT_SWITCH;
    d.cutoff = 12.0;
    d.cuton = 10.0;
    d.dcut = 2.0;
    d.temp = 300.0;
    d.precision = MCG_PREC_FP64;

    counts = (int*)malloc(sizeof(int) * (size_t)d.natom);
    if (!counts) return 4;
    report("build_exclusions", mcg_build_exclusions(&d, counts, NULL, 0, &total, NULL, 0, &n14));
    printf("excl_total %lld\n", (long long)total);
    printf("pairs14 %d\n", n14);
    free(counts);

    /* null arguments are rejected, not dereferenced */
    report("null_create", mcg_create(NULL, &s));
    report("null_energy", mcg_energy(NULL, ener));

    rc = report("create", mcg_create(&d, &s));
    if (rc == MCG_OK) {
        int atoms[1] = {0};
        double nx[1], ny[1], nz[1], de = 0.0;
        nx[0] = d.x[0] + 0.05;
        ny[0] = d.y[0];
        nz[0] = d.z[0];
        report("energy", mcg_energy(s, ener));
        printf("etot %.17g\n", ener[0]);
        report("delta_e", mcg_delta_e(s, 1, atoms, nx, ny, nz, &de));
        printf("de %.17g\n", de);
        report("destroy", mcg_destroy(s));
    }
    o.dmax_trn = 0.15;
    o.dmax_rot = 15.0;
    o.acceptance_units = MCG_ACCEPT_PHYSICAL;
    o.seed = 1;
    if (mcg_device_count() == 0) report("batch_create", mcg_batch_create(&d, 1, &o, &b));
    report("mdbas_free", mcg_mdbas_free(m));
    return 0;
}
