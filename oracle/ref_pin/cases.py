"""Cases for the reference pin (TEST INFRASTRUCTURE ONLY).

The reference bakes its case into the device code through parameters.h macros (LX, LY, LZ, RHO0,
REP_STF*, ...), so its kernels are compiled once per case.  Each case is a set of parameters.h
values; the same values configure the oracle and librbtp in tests/test_gpu_ref_pin.py.
"""
import math

CASES = {
    # single phase, 32x32x16, Ra = 1e6
    "ref_single": dict(lx=32, ly=32, lz=16, rayleigh=1.0e6, prandtl=0.71,
                       visc=0.1414 * 32 * math.sqrt(0.71 / 1.0e6), activate_particles=0,
                       particle_fraction=0.0, particle_diam_frac=1.0 / 20.0,
                       rho_particle_ratio=1.0),
    # the plain FP64 parity configuration: 64x64x32, Ra = 1e6, single phase
    "ref_config1": dict(lx=64, ly=64, lz=32, rayleigh=1.0e6, prandtl=0.71,
                        visc=0.1414 * 64 * math.sqrt(0.71 / 1.0e6), activate_particles=0,
                        particle_fraction=0.0, particle_diam_frac=1.0 / 20.0,
                        rho_particle_ratio=1.0),
    # nine spheres of diameter 8 in 48x48x24
    "ref_particles": dict(lx=48, ly=48, lz=24, rayleigh=1.0e6, prandtl=0.71,
                          visc=0.1414 * 48 * math.sqrt(0.71 / 1.0e6), activate_particles=1,
                          particle_fraction=0.04, particle_diam_frac=8.0 / 48.0,
                          rho_particle_ratio=1.0),
}

# Timing cases (oracle/ref_pin/time_ref.py): the benchmark workloads, 320x320x160 at Ra = 1e8,
# single phase and with 1000 spheres of diameter 16 at density ratio 1.0.
_V16 = 4.0 * math.pi * 8.0 ** 3 / 3.0
TIMING = {
    "ref_production": dict(lx=320, ly=320, lz=160, rayleigh=1.0e8, prandtl=0.71,
                           visc=0.1414 * 320 * math.sqrt(0.71 / 1.0e8), activate_particles=0,
                           particle_fraction=0.0, particle_diam_frac=1.0 / 20.0,
                           rho_particle_ratio=1.0),
    "ref_particle_laden": dict(lx=320, ly=320, lz=160, rayleigh=1.0e8, prandtl=0.71,
                               visc=0.1414 * 320 * math.sqrt(0.71 / 1.0e8), activate_particles=1,
                               particle_fraction=1000.5 * _V16 / (320 * 320 * 160),
                               particle_diam_frac=16.0 / 320.0, rho_particle_ratio=1.0),
}

# parameters.h macros that are not case fields (reference defaults, parameters.h:4-53)
FIXED = dict(continuous_steps=0, nend=1000000, ndiag=125, nflowout=25000, nnuout=125, nout_p=125,
             t_hot=1.0, t_cold=0.0, t_ref=0.5, beta=0.0000625, rho0=1.0, cp_particle_ratio=10.0,
             cp_fluid=1.0, repforce_scale=2.0e-4, particle_init_temp=0.5, particle_rand_seed=86143,
             rep_min_gap=2.0, rep_min_gap_w=2.0, rep_stf0=0.025, rep_stf1=0.002, rep_stf0_w=0.025,
             rep_stf1_w=0.002)


def values(case: str, **over) -> dict:
    """parameters.h values of a case.  Overrides may change what the compiled kernels take at run
    time (Ra, Pr and VISC enter only through the constants the driver sets; the density ratio only
    through the particle mass and the integrator's argument), not the compiled sizes."""
    v = dict(FIXED)
    v.update(CASES[case] if case in CASES else TIMING[case])
    v.update(over)
    return v


def parameters_h(case: str) -> str:
    v = values(case)
    d = lambda x: repr(float(x))  # noqa: E731  (full-precision double literal)
    return f"""#ifndef PARAMETERS_H
#define PARAMETERS_H
#define CONTINUOUS_STEPS {v['continuous_steps']}
#define LX {v['lx']}
#define LY {v['ly']}
#define LZ {v['lz']}
#define LXY (LX * LY)
#define LXYZ (LX * LY * LZ)
#define NPOP 27
#define NEND {v['nend']}
#define NDIAG {v['ndiag']}
#define NFLOWOUT {v['nflowout']}
#define NNUOUT {v['nnuout']}
#define NOUT_P {v['nout_p']}
#define RAYLEIGH {d(v['rayleigh'])}
#define PRANDTL {d(v['prandtl'])}
#define T_HOT {d(v['t_hot'])}
#define T_COLD {d(v['t_cold'])}
#define T_REF {d(v['t_ref'])}
#define BETA {d(v['beta'])}
#define VISC {d(v['visc'])}
#define RHO0 {d(v['rho0'])}
#define ACTIVATE_PARTICLES {v['activate_particles']}
#define PARTICLE_FRACTION {d(v['particle_fraction'])}
#define PARTICLE_DIAM_FRAC ({d(v['particle_diam_frac'])})
#define CP_PARTICLE_RATIO {d(v['cp_particle_ratio'])}
#define CP_FLUID {d(v['cp_fluid'])}
#define RHO_PARTICLE_RATIO {d(v['rho_particle_ratio'])}
#define REPFORCE_SCALE {d(v['repforce_scale'])}
#define PARTICLE_INIT_TEMP {d(v['particle_init_temp'])}
#define PARTICLE_RAND_SEED {v['particle_rand_seed']}
#define REP_MIN_GAP {d(v['rep_min_gap'])}
#define REP_MIN_GAP_W {d(v['rep_min_gap_w'])}
#define REP_STF0 {d(v['rep_stf0'])}
#define REP_STF1 {d(v['rep_stf1'])}
#define REP_STF0_W {d(v['rep_stf0_w'])}
#define REP_STF1_W {d(v['rep_stf1_w'])}
#define BLOCK_X 8
#define BLOCK_Y 8
#define BLOCK_Z 4
#endif
"""
