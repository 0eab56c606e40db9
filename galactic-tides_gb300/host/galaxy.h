/*
 * Synthetic galaxies for benchmarks and tests (libgtc_ics.so).
 *
 * A disk + bulge + halo galaxy after Hernquist (1993), the benchmark input
 * of the reference (make_hernquist_galaxy, src/hernquist_ics.cpp:142). The
 * positions and masses are those the reference draws for the same model and
 * seed -- same generator (std::mt19937_64), same draws in the same order,
 * same profile tables and inversions -- so a run here and a run of the
 * reference start from the same particles (bit for bit where the C library's
 * exp/log/sin/cos agree, which they do on x86-64 glibc).
 *
 * Velocities follow the reference's moment equations (spherical Jeans
 * equation for bulge and halo with escape-speed truncation, isothermal sheet
 * and Toomre-Q normalised dispersions with the epicyclic approximation and
 * asymmetric drift for the disk) but take the radial force and potential
 * from the analytic enclosed mass, where the reference measures them with its
 * own tree on the realised particles. They are a plausible equilibrium for
 * integration tests, not the reference's values.
 */
#ifndef GTC_GALAXY_H
#define GTC_GALAXY_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* HernquistModel (include/galactic_tides/hernquist_ics.h:55-77). */
typedef struct gtc_galaxy_model {
  double G;
  uint64_t disk_n, bulge_n, halo_n;
  double disk_mass, disk_h, disk_z0, disk_rmax, disk_Q, disk_Q_radius;
  double bulge_mass, bulge_a, bulge_rmax;
  double halo_mass, halo_core, halo_cutoff, halo_rmax;
  double vesc_fraction;
  uint64_t seed;
} gtc_galaxy_model;

/* The benchmark galaxy of n particles: disk 40 % (M=1, h=1, z0=0.1), bulge
 * 13 % (M=0.33, a=0.2), halo the rest (M=5.8, core 1, cutoff 10); the other
 * fields at the reference's defaults. */
void gtc_galaxy_default(gtc_galaxy_model *m, uint64_t n, uint64_t seed);

/* Fills pos/vel (n x 3), mass (n), type (n: 1 halo, 2 disk, 3 bulge) for
 * n = halo_n + disk_n + bulge_n particles, halo first, then disk, then bulge,
 * centred on the centre of mass at rest. Returns 0, or 1 on a bad model. */
int gtc_make_galaxy(const gtc_galaxy_model *m, double *pos, double *vel, double *mass,
                    int32_t *type);

/* Rotates positions and velocities of n bodies by incl_deg about x, then
 * omega_deg about z (orient, src/hernquist_ics.cpp). */
void gtc_orient(double *pos, double *vel, uint64_t n, double incl_deg, double omega_deg);

/* Relative position dx and velocity dv of a parabolic two-point-mass orbit
 * with pericentre rp, approaching from separation r0 in the x-y plane
 * (parabolic_orbit, src/hernquist_ics.cpp). Returns 1 if r0 < rp. */
int gtc_parabolic_orbit(double G, double m1, double m2, double rp, double r0, double dx[3],
                        double dv[3]);

/* A parabolic encounter of two galaxies of model m (seeds m.seed and
 * m.seed + 1), inclined incl1 / incl2 degrees (omega1 / omega2 about z),
 * pericentre rp, start separation r0, centre of mass at rest at the origin:
 * the encounter mode of apps/galactic_tides_ics.cpp:78-97. Fills 2 n
 * bodies (n = one galaxy), galaxy 1 first. Returns 0, or 1 on a bad model
 * or orbit. */
int gtc_make_encounter(const gtc_galaxy_model *m, double incl1, double omega1, double incl2,
                       double omega2, double rp, double r0, double *pos, double *vel,
                       double *mass, int32_t *type);

/* The accuracy sample of the reference bench (apps/galactic_tides_bench.cpp:
 * 75-79): indices 0..n-1 shuffled by std::shuffle with std::mt19937_64(seed),
 * first m kept. */
void gtc_sample_indices(uint64_t n, uint64_t m, uint64_t seed, uint64_t *out);

#ifdef __cplusplus
}
#endif

#endif
