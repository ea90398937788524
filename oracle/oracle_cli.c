/*
 * oracle_cli.c -- command-line twin of the reference's `flock-ref` tool
 * (crates/flock-ref/src/main.rs:11-80), over the C oracle. Test
 * infrastructure: the parity ladder in tests/ drives it beside the product CLI.
 *
 *   flock_ref_c gen   --birds N [--seed S] --out FILE
 *   flock_ref_c step  --in FILE --steps K --out FILE
 *   flock_ref_c diff  A.flk B.flk [--pos-tol X] [--vel-tol X] [--allow-outliers N] [--outlier-max X]
 *   flock_ref_c stats FILE
 *   flock_ref_c statdiff A.flk B.flk
 *
 * Exit codes follow main.rs:18-27,128-132: 0 pass, 1 parity failure, 2 usage/IO.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "flock_oracle.h"

static const char* USAGE =
    "usage:\n"
    "  flock_ref_c gen   --birds N [--seed S] --out FILE\n"
    "  flock_ref_c step  --in FILE --steps K --out FILE     (brute force; use N <= ~5000)\n"
    "  flock_ref_c diff  A.flk B.flk [--pos-tol X] [--vel-tol X] [--allow-outliers N] [--outlier-max X]\n"
    "  flock_ref_c stats FILE\n"
    "  flock_ref_c statdiff A.flk B.flk     (aggregate agreement for long, chaotic runs)\n";

static const char* opt(int argc, char** argv, const char* name) {
    for (int k = 1; k + 1 < argc; ++k)
        if (strcmp(argv[k], name) == 0) return argv[k + 1];
    return NULL;
}

static int fail(const char* msg) {
    fprintf(stderr, "flock_ref_c: %s\n\n%s", msg, USAGE);
    return 2;
}

static orc_bird* load(const char* path, uint32_t* n, float* time) {
    if (orc_read_header(path, n, time) != 0) return NULL;
    orc_bird* b = (orc_bird*)malloc(sizeof(orc_bird) * (*n ? *n : 1));
    if (orc_read_flk(path, time, b, *n) != 0) { free(b); return NULL; }
    return b;
}

int main(int argc, char** argv) {
    if (argc < 2) return fail("missing or unknown command");
    const char* cmd = argv[1];
    if (strcmp(cmd, "gen") == 0) {
        const char* nb = opt(argc, argv, "--birds");
        const char* seed = opt(argc, argv, "--seed");
        const char* out = opt(argc, argv, "--out");
        if (!nb) return fail("missing --birds");
        if (!out) return fail("missing --out");
        uint32_t n = (uint32_t)strtoul(nb, NULL, 10);
        orc_bird* b = (orc_bird*)malloc(sizeof(orc_bird) * (n ? n : 1));
        orc_scatter(n, seed ? strtoull(seed, NULL, 10) : 1ull, b);
        int rc = orc_write_flk(out, 0.0f, b, n);
        free(b);
        return rc ? fail("cannot write --out") : 0;
    }
    if (strcmp(cmd, "step") == 0) {
        const char* in = opt(argc, argv, "--in");
        const char* ks = opt(argc, argv, "--steps");
        const char* out = opt(argc, argv, "--out");
        if (!in) return fail("missing --in");
        if (!ks) return fail("missing --steps");
        if (!out) return fail("missing --out");
        uint32_t n;
        float time;
        orc_bird* b = load(in, &n, &time);
        if (!b) return fail("cannot read --in");
        long k = strtol(ks, NULL, 10);
        for (long s = 0; s < k; ++s) time = orc_step(b, n, time, NULL, NULL, 0);
        int rc = orc_write_flk(out, time, b, n);
        free(b);
        return rc ? fail("cannot write --out") : 0;
    }
    if (strcmp(cmd, "stats") == 0) {
        if (argc < 3) return fail("missing FILE");
        uint32_t n;
        float time;
        orc_bird* b = load(argv[2], &n, &time);
        if (!b) return fail("cannot read FILE");
        float s[4];
        orc_stats(b, n, s);
        printf("birds %u  time %.3f s\n", n, time);
        printf("mean speed %.4f m/s  mean neighbours %.3f  mean radius %.3f m  polarization %.4f\n", s[0], s[1], s[2], s[3]);
        free(b);
        return 0;
    }
    if (strcmp(cmd, "diff") == 0 || strcmp(cmd, "statdiff") == 0) {
        if (argc < 4) return fail("missing A or B");
        uint32_t na, nb;
        float ta, tb;
        orc_bird* a = load(argv[2], &na, &ta);
        orc_bird* b = load(argv[3], &nb, &tb);
        if (!a || !b) return fail("cannot read A or B");
        if (na != nb) return fail("files hold different bird counts");
        int ok;
        if (strcmp(cmd, "statdiff") == 0) {
            float d[4], sa[4], sb[4];
            const float tol[4] = {0.02f, 0.1f, 0.01f, 0.005f};
            const char* names[4] = {"mean speed", "mean neighbours", "mean radius", "polarization"};
            ok = orc_statdiff(a, b, na, d);
            orc_stats(a, na, sa);
            orc_stats(b, nb, sb);
            for (int k = 0; k < 4; ++k)
                printf("%-16s A %9.4f  B %9.4f  |d| %.4f  (tol %g)\n", names[k], sa[k], sb[k], d[k], tol[k]);
        } else {
            const char* pt = opt(argc, argv, "--pos-tol");
            const char* vt = opt(argc, argv, "--vel-tol");
            const char* al = opt(argc, argv, "--allow-outliers");
            const char* om = opt(argc, argv, "--outlier-max");
            float out[7];
            uint32_t mism, outl;
            uint32_t allow = al ? (uint32_t)strtoul(al, NULL, 10) : 0u;
            float omax = om ? strtof(om, NULL) : 1e-2f;
            ok = orc_diff(a, b, na, pt ? strtof(pt, NULL) : 1e-3f, vt ? strtof(vt, NULL) : 1e-3f, allow, omax, out, &mism,
                          &outl);
            printf("birds %u  time A %.4f B %.4f\n", na, ta, tb);
            printf("max |dpos| %.3e  max |dvel| %.3e  max |dradius| %.3e  max |dcentrality| %.3e\n", out[0], out[1], out[2],
                   out[3]);
            printf("neighbour-count mismatches %u of %u\n", mism, na);
            printf("(informational) max |dsteering| %.3e  max |droll| %.3e  max |dspin| %.3e\n", out[4], out[5], out[6]);
            if (allow > 0) printf("birds above tolerance: %u (allowed %u, each below %g)\n", outl, allow, omax);
        }
        printf("%s\n", ok ? "PASS" : "FAIL");
        free(a);
        free(b);
        return ok ? 0 : 1;
    }
    return fail("missing or unknown command");
}
