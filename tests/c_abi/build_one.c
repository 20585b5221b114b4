/* build_one.c - the C ABI from C: one atmosphere with the crate's default
 * parameters (Parameters::default, src/precompute.rs:849-935), built, waited
 * for, its three tables copied to host memory; prints one line with the
 * table sizes and the sums of their RGB channels. Exit status 0 on success.
 * Compiled with -std=c11 -pedantic by the tests: include/fuzzyblue.h is plain C.
 *
 * usage: build_one [order] [precision]   (defaults: 4, 0 = plain FP32) */
#include <stdio.h>
#include <stdlib.h>

#include "fuzzyblue.h"

static int check(int status, const char* what) {
    if (status < 0) fprintf(stderr, "%s: %s (%s)\n", what, fb_status_string(status), fb_last_error());
    return status < 0;
}

static double rgb_sum(const float* t, size_t texels) {
    double s = 0.0;
    for (size_t i = 0; i < texels; ++i) s += (double)t[4 * i] + t[4 * i + 1] + t[4 * i + 2];
    return s;
}

int main(int argc, char** argv) {
    fb_params p;
    fb_extent tr, ir, sc;
    fb_builder* b = NULL;
    fb_pending* pend = NULL;
    fb_atmosphere* atm = NULL;
    float *t = NULL, *i = NULL, *s = NULL;
    size_t nt, ni, ns;
    int rc = 1;

    fb_params_default(&p);
    if (argc > 1) p.order = (uint32_t)atoi(argv[1]);
    if (argc > 2) p.precision = (uint32_t)atoi(argv[2]);
    if (check(fb_params_extents(&p, &tr, &ir, &sc), "fb_params_extents")) return 1;
    nt = (size_t)tr.width * tr.height;
    ni = (size_t)ir.width * ir.height;
    ns = (size_t)sc.width * sc.height * sc.depth;
    t = (float*)malloc(16 * nt);
    i = (float*)malloc(16 * ni);
    s = (float*)malloc(16 * ns);
    if (!t || !i || !s) goto done;
    if (check(fb_builder_create(0, &b), "fb_builder_create")) goto done;
    if (check(fb_atmosphere_build(b, NULL, &p, &pend), "fb_atmosphere_build")) goto done;
    if (check(fb_pending_take(pend, 0, &atm), "fb_pending_take")) goto done;
    if (check(fb_atmosphere_copy_to_host(atm, NULL, t, i, s), "fb_atmosphere_copy_to_host")) goto done;
    printf("transmittance %ux%u irradiance %ux%u scattering %ux%ux%u sums %.9e %.9e %.9e\n", tr.width, tr.height,
           ir.width, ir.height, sc.width, sc.height, sc.depth, rgb_sum(t, nt), rgb_sum(i, ni), rgb_sum(s, ns));
    rc = 0;
done:
    if (atm) fb_atmosphere_destroy(atm);
    if (pend) fb_pending_release(pend);
    if (b) fb_builder_destroy(b);
    free(t);
    free(i);
    free(s);
    return rc;
}
