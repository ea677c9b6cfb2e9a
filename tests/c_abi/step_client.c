/* A plain C client of libmfem_gb300: builds a plan from a mesh file, runs
 * steps on device buffers it allocates itself, and writes the positions.
 * Used by tests/test_gpu_c_client.py to show the C ABI needs nothing but the
 * header, the library and the CUDA runtime.
 *
 * Mesh file (little endian): int32 n, T, steps, energy; float32 dt;
 * float32 rest[n][3], mass[n], inv_mass[n]; int32 tets[T][4];
 * float32 poses[T][9], materials[T][3], gravity[3].
 * Output file: float32 q[n][3] after the steps, then int32 PCG iterations of
 * the last step's Newton iterations.
 * Exit code 0 on success. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime_api.h>

#include "mfem_gb300.h"

static int read_all(FILE *f, void *dst, size_t bytes) { return fread(dst, 1, bytes, f) == bytes; }

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s mesh.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t head[4];
    float dt;
    if (!read_all(f, head, sizeof(head)) || !read_all(f, &dt, sizeof(dt))) return 4;
    const int32_t n = head[0], T = head[1], steps = head[2], energy = head[3];
    float *rest = malloc(sizeof(float) * 3 * n), *mass = malloc(sizeof(float) * n);
    float *inv_mass = malloc(sizeof(float) * n), *poses = malloc(sizeof(float) * 9 * T);
    float *materials = malloc(sizeof(float) * 3 * T), gravity[3];
    int32_t *tets = malloc(sizeof(int32_t) * 4 * T);
    if (!read_all(f, rest, sizeof(float) * 3 * n) || !read_all(f, mass, sizeof(float) * n) ||
        !read_all(f, inv_mass, sizeof(float) * n) || !read_all(f, tets, sizeof(int32_t) * 4 * T) ||
        !read_all(f, poses, sizeof(float) * 9 * T) || !read_all(f, materials, sizeof(float) * 3 * T) ||
        !read_all(f, gravity, sizeof(gravity)))
        return 5;
    fclose(f);

    mfem_config cfg;
    mfem_config_default(&cfg);
    cfg.energy = energy;
    mfem_plan *plan = NULL;
    int rc = mfem_plan_create(&cfg, n, T, tets, poses, materials, rest, mass, inv_mass, gravity, 0, &plan);
    if (rc != MFEM_OK) {
        fprintf(stderr, "mfem_plan_create: %s\n", mfem_plan_last_error(NULL));
        return 6;
    }
    float *q[2], *qd[2];
    for (int i = 0; i < 2; ++i) {
        if (cudaMalloc((void **)&q[i], sizeof(float) * 3 * n) != cudaSuccess) return 7;
        if (cudaMalloc((void **)&qd[i], sizeof(float) * 3 * n) != cudaSuccess) return 7;
    }
    cudaMemcpy(q[0], rest, sizeof(float) * 3 * n, cudaMemcpyHostToDevice);
    cudaMemset(qd[0], 0, sizeof(float) * 3 * n);
    int cur = 0;
    for (int s = 0; s < steps; ++s) {
        rc = mfem_step(plan, q[cur], qd[cur], q[1 - cur], qd[1 - cur], dt, NULL);
        if (rc != MFEM_OK) {
            fprintf(stderr, "mfem_step: %s\n", mfem_plan_last_error(plan));
            return 8;
        }
        cur = 1 - cur;
    }
    mfem_solve_stats stats[64];
    int32_t count = 0;
    rc = mfem_step_stats(plan, stats, 64, &count, NULL);
    if (rc != MFEM_OK) return 9;
    float *out = malloc(sizeof(float) * 3 * n);
    if (cudaMemcpy(out, q[cur], sizeof(float) * 3 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 10;
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 11;
    fwrite(out, sizeof(float), 3 * (size_t)n, o);
    for (int i = 0; i < count; ++i) fwrite(&stats[i].iterations, sizeof(int32_t), 1, o);
    fclose(o);
    mfem_plan_destroy(plan);
    for (int i = 0; i < 2; ++i) {
        cudaFree(q[i]);
        cudaFree(qd[i]);
    }
    free(rest);
    free(mass);
    free(inv_mass);
    free(poses);
    free(materials);
    free(tets);
    free(out);
    return 0;
}
