/* Case macros of the drop-in host rb3d: the same names and meaning as the reference's
 * parameters.h (parameters.h:1-55).  Edit and rebuild, as with the reference.  BLOCK_X/Y/Z are
 * accepted for source compatibility; librbtp chooses its own launch shapes. */
#ifndef PARAMETERS_H
#define PARAMETERS_H

// Continue calculation
#define CONTINUOUS_STEPS 0

// Grid dimensions
#define LX 320
#define LY 320
#define LZ 160
#define LXY (LX * LY)
#define LXYZ (LX * LY * LZ)
#define NPOP 27

// Time steps
#define NEND 1000000
#define NDIAG 125
#define NFLOWOUT 25000
#define NNUOUT 125
#define NOUT_P 125

// Physical parameters
#define RAYLEIGH 1.0e7
#define PRANDTL 0.71
#define T_HOT 1.0
#define T_COLD 0.0
#define T_REF 0.5
#define BETA 0.0000625
#define VISC 0.01206
#define RHO0 1.0

// Particle controls
#define ACTIVATE_PARTICLES 1
#define PARTICLE_FRACTION 0.05
#define PARTICLE_DIAM_FRAC (1.0/20.0)
#define CP_PARTICLE_RATIO 10.0
#define CP_FLUID 1.0
#define RHO_PARTICLE_RATIO 1.0
#define REPFORCE_SCALE 2.0e-4
#define PARTICLE_INIT_TEMP (T_COLD + T_HOT)/2

#define PARTICLE_RAND_SEED 86143
#define REP_MIN_GAP 2.0
#define REP_MIN_GAP_W 2.0
#define REP_STF0 0.025
#define REP_STF1 0.002
#define REP_STF0_W 0.025
#define REP_STF1_W 0.002

// Block dimensions (ignored by librbtp)
#define BLOCK_X 8
#define BLOCK_Y 8
#define BLOCK_Z 4

// librbtp extension: population storage (0 = FP64, 1 = FP32, 2 = shifted FP16)
#ifndef RBTP_STORAGE
#define RBTP_STORAGE 0
#endif

#endif
