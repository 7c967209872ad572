/*
 * A plain C client of libpfgb300.so: K explicit Euler steps of the phase
 * field with a temperature array (pfg_pf_step), no Python involved.
 *
 *   pf_client <params.bin> <eta0.bin> <T.bin> <steps> <dt> <eta_out.bin>
 *
 * params.bin holds one pfg_pf_params struct as the library lays it out
 * (pfg_struct_size(0) bytes), eta0.bin N * num_oris float32, T.bin N float32.
 * Exit status 0 on success; the library's status string on failure.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

#include "pf_gb300.h"

static void* read_file(const char* path, size_t bytes) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  void* buf = malloc(bytes);
  if (buf && fread(buf, 1, bytes, f) != bytes) {
    free(buf);
    buf = NULL;
  }
  fclose(f);
  return buf;
}

int main(int argc, char** argv) {
  if (argc != 7) {
    fprintf(stderr, "usage: %s params.bin eta0.bin T.bin steps dt eta_out.bin\n", argv[0]);
    return 2;
  }
  if (pfg_struct_size(0) != (int64_t)sizeof(pfg_pf_params)) {
    fprintf(stderr, "pfg_pf_params size mismatch\n");
    return 3;
  }
  pfg_pf_params* p = (pfg_pf_params*)read_file(argv[1], sizeof(pfg_pf_params));
  if (!p) return 4;
  const int n = p->num_oris;
  const size_t N = (size_t)p->nx * p->ny * p->nz, NN = N * (size_t)n;
  float* eta_h = (float*)read_file(argv[2], NN * sizeof(float));
  float* T_h = (float*)read_file(argv[3], N * sizeof(float));
  if (!eta_h || !T_h) return 5;
  const int steps = atoi(argv[4]);
  const float dt = (float)atof(argv[5]);
  float *eta_a = NULL, *eta_b = NULL, *T_d = NULL;
  if (cudaMalloc((void**)&eta_a, NN * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void**)&eta_b, NN * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void**)&T_d, N * sizeof(float)) != cudaSuccess)
    return 6;
  cudaMemcpy(eta_a, eta_h, NN * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(T_d, T_h, N * sizeof(float), cudaMemcpyHostToDevice);
  for (int k = 0; k < steps; ++k) {
    const int st = pfg_pf_step(p, eta_a, eta_b, T_d, dt, NULL);
    if (st != PFG_OK) {
      fprintf(stderr, "pfg_pf_step: %s (%s)\n", pfg_status_string(st), pfg_last_cuda_error());
      return 7;
    }
    float* t = eta_a;
    eta_a = eta_b;
    eta_b = t;
  }
  if (cudaDeviceSynchronize() != cudaSuccess || pfg_device_error(1) != 0) return 8;
  cudaMemcpy(eta_h, eta_a, NN * sizeof(float), cudaMemcpyDeviceToHost);
  FILE* f = fopen(argv[6], "wb");
  if (!f || fwrite(eta_h, sizeof(float), NN, f) != NN) return 9;
  fclose(f);
  cudaFree(eta_a);
  cudaFree(eta_b);
  cudaFree(T_d);
  free(eta_h);
  free(T_h);
  free(p);
  printf("pf_client: %d steps of %zu cells x %d orientations\n", steps, N, n);
  return 0;
}
