/*
 * A plain C caller of the drop-in entry point, as an application linking
 * libcutcint.so would be (the reference documents C/C++ callers in its
 * README, and src/cutc_int_f.f90 is its Fortran demo).  Reads the inputs of
 * one problem from raw files, calls cutc_int with the reference's argument
 * list, writes X and int_2e, and prints the status.
 *
 *   call_cutc_int <dir> <n_grid1> <n_grid2> <n_ao> <n_nuc> <size_bh>
 * <dir> holds r1.bin wr1.bin r2.bin wr2.bin rn.bin aos1.bin aos2.bin c_bh.bin
 * m_bh.bin n_bh.bin o_bh.bin (native doubles / int32, Fortran order); the
 * outputs go to X.bin and int2e.bin in the same directory.
 */
#include <stdio.h>
#include <stdlib.h>

#include "cutc_int.h"

static void *load(const char *dir, const char *name, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    void *p = malloc(bytes ? bytes : 1);
    if (!f || !p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot read %s\n", path);
        exit(2);
    }
    fclose(f);
    return p;
}

static void save(const char *dir, const char *name, const void *p, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: %s dir n_grid1 n_grid2 n_ao n_nuc size_bh\n", argv[0]);
        return 2;
    }
    const char *dir = argv[1];
    const int n1 = atoi(argv[2]), n2 = atoi(argv[3]), na = atoi(argv[4]);
    const int nn = atoi(argv[5]), nb = atoi(argv[6]);
    const size_t d = sizeof(double), i = sizeof(int);
    double *r1 = load(dir, "r1.bin", 3 * (size_t)n1 * d);
    double *wr1 = load(dir, "wr1.bin", (size_t)n1 * d);
    double *r2 = load(dir, "r2.bin", 3 * (size_t)n2 * d);
    double *wr2 = load(dir, "wr2.bin", (size_t)n2 * d);
    double *rn = load(dir, "rn.bin", 3 * (size_t)nn * d);
    double *aos1 = load(dir, "aos1.bin", 4 * (size_t)n1 * na * d);
    double *aos2 = load(dir, "aos2.bin", 4 * (size_t)n2 * na * d);
    double *c = load(dir, "c_bh.bin", (size_t)nb * nn * d);
    int *m = load(dir, "m_bh.bin", (size_t)nb * nn * i);
    int *n = load(dir, "n_bh.bin", (size_t)nb * nn * i);
    int *o = load(dir, "o_bh.bin", (size_t)nb * nn * i);
    const size_t xs = 3 * (size_t)n1 * na * na, is = (size_t)na * na * na * na;
    double *X = malloc(xs * d), *I = malloc(is * d);
    /* launch geometry of the reference demo (src/cutc_int_f.f90:13-14): accepted and ignored */
    int s = cutc_int(100, 32, 1, 32, 1, 1, n1, n2, na, nn, nb, r1, wr1, r2, wr2, rn, aos1, aos2,
                     c, m, n, o, X, I);
    printf("status %d\n", s);
    if (s != 0) {
        printf("%s\n", cutc_last_error());
        return 1;
    }
    save(dir, "X.bin", X, xs * d);
    save(dir, "int2e.bin", I, is * d);
    return 0;
}
