/* c_abi_client.c -- a plain C99 client of the engine's C ABI (include/swit_gb300.h),
 * as a host program outside Python would use it: describe a survey, create an
 * engine, set the model, and run a Waveform-misfit gradient with host buffers.
 *
 *   c_abi_client invalid   create with a bad description: must fail with
 *                          SWIT_E_ARG before any GPU work (no GPU needed)
 *   c_abi_client           the whole gradient on a small layered model (GPU)
 *
 * Exit status 0 when the calls behave as documented. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swit_gb300.h"

enum { NX = 48, NZ = 32, NPML = 10, NT = 300, NS = 2, NG = 48 };

int main(int argc, char** argv) {
  static int32_t ng[NS];
  static float sx[NS], sz[NS], gx[NS * NG], gz[NS * NG];
  for (int s = 0; s < NS; ++s) {
    ng[s] = NG;
    sx[s] = 100.0f + 200.0f * (float)s;
    sz[s] = 20.0f;
    for (int g = 0; g < NG; ++g) {
      gx[s * NG + g] = 10.0f * (float)g;
      gz[s * NG + g] = 10.0f;
    }
  }
  swit_desc d;
  memset(&d, 0, sizeof d); /* every option 0: FP32, batched, automatic */
  d.nx = NX;
  d.nz = NZ;
  d.npml = NPML;
  d.nt = NT;
  d.dx = 10.0f;
  d.dt = 0.001f;
  d.free_surface = 1;
  d.ns = NS;
  d.ng_max = NG;
  d.ng = ng;
  d.src_x = sx;
  d.src_z = sz;
  d.rec_x = gx;
  d.rec_z = gz;
  swit_engine* e = NULL;

  if (argc > 1 && strcmp(argv[1], "invalid") == 0) {
    d.nx = 4; /* below the minimum grid */
    const int rc = swit_create(&d, &e);
    printf("swit_create: %d (%s)\n", rc, swit_last_error());
    return (rc == SWIT_E_ARG && e == NULL && strlen(swit_last_error()) > 0) ? 0 : 1;
  }

  int rc = swit_create(&d, &e);
  if (rc) {
    fprintf(stderr, "swit_create: %s\n", swit_last_error());
    return 1;
  }
  static float vp[NX * NZ], vp0[NX * NZ], rho[NX * NZ], src[NS * NT];
  for (int ix = 0; ix < NX; ++ix)
    for (int iz = 0; iz < NZ; ++iz) {
      const int k = ix * NZ + iz; /* z-fastest, nx records of nz */
      vp[k] = 1800.0f + 1400.0f * (float)iz / (float)(NZ - 1);
      vp0[k] = vp[k] * 0.97f;
      rho[k] = 310.0f * powf(vp[k], 0.25f);
    }
  for (int s = 0; s < NS; ++s)
    for (int it = 0; it < NT; ++it) {
      const float t = (float)it * 0.001f - 0.048f, a = 3.14159265f * 25.0f * t;
      src[s * NT + it] = t * expf(-a * a); /* an integrated Ricker-like pulse */
    }
  static float obs[NS * NG * NT], grad[NX * NZ], fw[NX * NZ], bk[NX * NZ];
  double misfit = 0.0;
  if ((rc = swit_set_model(e, vp, rho, 0, NULL)) || (rc = swit_forward(e, src, obs, 0, 0, NULL)) ||
      (rc = swit_set_model(e, vp0, rho, 0, NULL)) ||
      (rc = swit_gradient_l2(e, src, obs, grad, fw, bk, NULL, &misfit, 0, NULL))) {
    fprintf(stderr, "engine call failed (%d): %s\n", rc, swit_last_error());
    swit_destroy(e);
    return 1;
  }
  double gn = 0.0;
  for (int k = 0; k < NX * NZ; ++k) gn += (double)grad[k] * grad[k];
  printf("misfit %.6e  |grad| %.6e\n", misfit, sqrt(gn));
  swit_destroy(e);
  return (misfit > 0.0 && gn > 0.0) ? 0 : 1;
}
