/* A plain C11 host of the zsmpm C ABI: the calls a zeno node (or any FFI
 * binding) makes for one scene, with no C++ and no Python in the process.
 *
 *   c_abi_driver <input> <output> <substeps>
 *
 * input (native endianness): int32 block_lo[3], block_dims[3]; boundary
 * int32 type, thickness, lo[3], hi[3]; material int32 type, plasticity,
 * float E, nu, density, friction_angle_deg, bulk, gamma; float dx, dt,
 * gravity[3]; int64 n; float x[3n], v[3n], m[n], vol[n].
 * output: int32 status of mpm_sync, then float x[3n], v[3n].
 * Exit status 0 on success, 1 on a usage or file error, 2 on an ABI error
 * (its text on stderr). */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "zsmpm.h"

static int rd(FILE *f, void *p, size_t size, size_t count) {
  return fread(p, size, count, f) == count;
}

static int fail(const char *what, int32_t rc) {
  fprintf(stderr, "%s failed (%d): %s\n", what, (int)rc, mpm_last_error());
  return 2;
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s <input> <output> <substeps>\n", argv[0]);
    return 1;
  }
  FILE *in = fopen(argv[1], "rb");
  if (!in) return 1;
  mpm_ctx_desc desc = {0};
  mpm_boundary bc;
  mpm_material mat;
  float dx, dt, gravity[3];
  int64_t n;
  int ok = rd(in, desc.block_lo, 4, 3) && rd(in, desc.block_dims, 4, 3) &&
           rd(in, &bc.type, 4, 1) && rd(in, &bc.thickness, 4, 1) && rd(in, bc.lo, 4, 3) &&
           rd(in, bc.hi, 4, 3) && rd(in, &mat.type, 4, 1) && rd(in, &mat.plasticity, 4, 1) &&
           rd(in, &mat.E, 4, 1) && rd(in, &mat.nu, 4, 1) && rd(in, &mat.density, 4, 1) &&
           rd(in, &mat.friction_angle_deg, 4, 1) && rd(in, &mat.bulk, 4, 1) &&
           rd(in, &mat.gamma, 4, 1) && rd(in, &dx, 4, 1) && rd(in, &dt, 4, 1) &&
           rd(in, gravity, 4, 3) && rd(in, &n, 8, 1);
  if (!ok || n <= 0) {
    fclose(in);
    return 1;
  }
  float *x = malloc(sizeof(float) * 3 * n), *v = malloc(sizeof(float) * 3 * n);
  float *m = malloc(sizeof(float) * n), *vol = malloc(sizeof(float) * n);
  ok = x && v && m && vol && rd(in, x, 4, 3 * n) && rd(in, v, 4, 3 * n) && rd(in, m, 4, n) &&
       rd(in, vol, 4, n);
  fclose(in);
  if (!ok) return 1;

  desc.device = 0;
  desc.dx = dx;
  desc.max_particles = n;
  mpm_ctx *ctx = NULL;
  int32_t rc;
  if ((rc = mpm_ctx_create(&desc, &ctx)) != MPM_OK) return fail("mpm_ctx_create", rc);
  if ((rc = mpm_set_materials(ctx, &mat, 1)) != MPM_OK) return fail("mpm_set_materials", rc);
  if ((rc = mpm_set_boundary(ctx, &bc)) != MPM_OK) return fail("mpm_set_boundary", rc);
  if ((rc = mpm_set_gravity(ctx, gravity[0], gravity[1], gravity[2])) != MPM_OK)
    return fail("mpm_set_gravity", rc);
  /* ToZSParticles defaults for the omitted arrays: C = 0, F = I, J = 1,
   * material 0 */
  rc = mpm_particles_upload(ctx, n, x, v, NULL, NULL, NULL, m, vol, NULL, NULL, NULL);
  if (rc != MPM_OK) return fail("mpm_particles_upload", rc);
  if ((rc = mpm_substep(ctx, dt, atoi(argv[3]))) != MPM_OK) return fail("mpm_substep", rc);
  const int32_t status = mpm_sync(ctx);
  if ((rc = mpm_particles_download(ctx, x, v, NULL, NULL, NULL)) != MPM_OK)
    return fail("mpm_particles_download", rc);
  mpm_ctx_destroy(ctx);

  FILE *out = fopen(argv[2], "wb");
  if (!out) return 1;
  ok = fwrite(&status, 4, 1, out) == 1 && fwrite(x, 4, 3 * n, out) == (size_t)(3 * n) &&
       fwrite(v, 4, 3 * n, out) == (size_t)(3 * n);
  fclose(out);
  free(x);
  free(v);
  free(m);
  free(vol);
  return ok ? 0 : 1;
}
