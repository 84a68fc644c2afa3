/*
 * ORACLE -- test infrastructure, never part of the product.
 *
 * CPU restatement, in plain C, of the MaHyCo per-cycle hydro hot path
 * (VNR and Eucclhyd Lagrange phases, directionally split remap, dual remap,
 * remap final, dt reduction) and of the reference initial states.  It keeps
 * the reference's data shapes (13-component conserved vectors per cell, face
 * arrays, n / n+1 buffer swaps) and its operation order, so that on the same
 * inputs it reproduces the reference bit for bit.  It is pinned against the
 * reference itself (oracle/_ref/mahyco_dump, built from the reference
 * sources) through the golden vectors in tests/golden/.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load it.
 */
#ifndef MAHYCO_PORT_H
#define MAHYCO_PORT_H
#include <stddef.h>

#include "../../include/hydro_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_run port_run;

/* Builds the mesh, runs the reference initialisation for spec->test_case and
 * returns a run positioned before cycle 1.  NULL on unsupported input (the
 * message is in port_last_error()). */
port_run* port_create(const hydro_spec* spec);
/* Runs up to ncycles cycles; returns cycles run, sets *done when the
 * reference loop condition ends the run. */
int port_step(port_run* r, int ncycles, int* done);
/* Field names: density pressure energy sound_speed pseudo divu cell_mass
 * density_env energy_env pressure_env fracvol_env mass_fraction_env (nc*3)
 * node_velocity (nn*2) node_mass cell_velocity (nc*2, Eucclhyd). */
int port_fetch(port_run* r, const char* field, double* dst, size_t n);
size_t port_field_size(port_run* r, const char* field);
int port_time(port_run* r, double* t, double* dt, long* cycle);
int port_error(port_run* r, unsigned* code, long* cell);
void port_destroy(port_run* r);
const char* port_last_error(void);
int port_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
