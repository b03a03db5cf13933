/*
 * A plain C caller that drives the reference's device-level stages itself, the
 * way the reference's own driver does (src/cutc_int.c:88-210): device buffers
 * from the CUDA runtime, get_int2_grad1_u12_ao with dim3 launch geometry
 * passed by value, then get_int_2e_ao.  The prototypes are written here with
 * CUDA's dim3, as a caller compiled against the reference's header has them,
 * and are resolved from libcutcint.so: the test is that such a caller links and
 * runs unchanged.  Reads and writes raw files like call_cutc_int.c; X comes
 * back with its four device components.
 *
 *   call_ref_stages <dir> <n_grid1> <n_grid2> <n_ao> <n_nuc> <size_bh>
 */
#include <cuda_runtime_api.h>
#include <stdio.h>
#include <stdlib.h>

const char *cutc_last_error(void);
void get_int2_grad1_u12_ao(dim3 dimGrid, dim3 dimBlock,
                           int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
                           double *r1, double *r2, double *wr2, double *rn, double *aos_data2,
                           double *c_bh, int *m_bh, int *n_bh, int *o_bh,
                           double *int2_grad1_u12_ao);
void get_int_2e_ao(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                   double *int2_grad1_u12, double *int_2e_ao);

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

/* host array -> new device array */
static void *to_dev(const void *h, size_t bytes)
{
    void *d = NULL;
    if (cudaMalloc(&d, bytes ? bytes : 1) != cudaSuccess ||
        cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        fprintf(stderr, "device copy failed\n");
        exit(3);
    }
    return d;
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
    double *r1 = to_dev(load(dir, "r1.bin", 3 * (size_t)n1 * d), 3 * (size_t)n1 * d);
    double *wr1 = to_dev(load(dir, "wr1.bin", (size_t)n1 * d), (size_t)n1 * d);
    double *r2 = to_dev(load(dir, "r2.bin", 3 * (size_t)n2 * d), 3 * (size_t)n2 * d);
    double *wr2 = to_dev(load(dir, "wr2.bin", (size_t)n2 * d), (size_t)n2 * d);
    double *rn = to_dev(load(dir, "rn.bin", 3 * (size_t)nn * d), 3 * (size_t)nn * d);
    double *aos1 = to_dev(load(dir, "aos1.bin", 4 * (size_t)n1 * na * d), 4 * (size_t)n1 * na * d);
    double *aos2 = to_dev(load(dir, "aos2.bin", 4 * (size_t)n2 * na * d), 4 * (size_t)n2 * na * d);
    double *c = to_dev(load(dir, "c_bh.bin", (size_t)nb * nn * d), (size_t)nb * nn * d);
    int *m = to_dev(load(dir, "m_bh.bin", (size_t)nb * nn * i), (size_t)nb * nn * i);
    int *n = to_dev(load(dir, "n_bh.bin", (size_t)nb * nn * i), (size_t)nb * nn * i);
    int *o = to_dev(load(dir, "o_bh.bin", (size_t)nb * nn * i), (size_t)nb * nn * i);
    const size_t xs = 4 * (size_t)n1 * na * na, is = (size_t)na * na * na * na;
    double *X = NULL, *I = NULL;
    if (cudaMalloc((void **)&X, xs * d) != cudaSuccess ||
        cudaMalloc((void **)&I, is * d) != cudaSuccess) {
        fprintf(stderr, "device allocation failed\n");
        return 3;
    }
    /* the reference driver's geometry for its pair kernel (src/cutc_int.c:42-48) */
    dim3 grid, block;
    grid.x = 100; grid.y = 32; grid.z = 1;
    block.x = 32; block.y = 1; block.z = 1;
    get_int2_grad1_u12_ao(grid, block, n1, n2, na, nn, nb, r1, r2, wr2, rn, aos2, c, m, n, o, X);
    get_int_2e_ao(n1, na, wr1, aos1, X, I);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        fprintf(stderr, "device error\n");
        return 3;
    }
    double *Xh = malloc(xs * d), *Ih = malloc(is * d);
    if (cudaMemcpy(Xh, X, xs * d, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(Ih, I, is * d, cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "copy back failed\n");
        return 3;
    }
    printf("last error: %s\n", cutc_last_error());
    save(dir, "X4.bin", Xh, xs * d);
    save(dir, "int2e.bin", Ih, is * d);
    return 0;
}
