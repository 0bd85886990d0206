/*
 * Compile-time configuration for building the reference code as an oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is force-included (-include) ahead
 * of the reference's own sources.  It defines the reference's include guard
 * `parameters_h` so that the reference's parameters.h becomes empty, and
 * then supplies every macro that parameters.h (parameters.h:41-366) defines,
 * with the same names and the same derived-quantity formulas, but with the
 * run-specific values taken from -D switches (ORC_*), so that one set of
 * reference sources can be built for several test configurations.
 *
 * The derived quantities (DX, DT, VTE, ...) must be the reference's own
 * formulas: they are interface, not implementation (parameters.h:75-262).
 */
#ifndef ORC_REF_PARAMS_H
#define ORC_REF_PARAMS_H
#define parameters_h 1
#define _CRT_SECURE_NO_WARNINGS

#include <stdio.h>
#include <iostream>
#include <stdlib.h>
#include <time.h>
#include <math.h>
#include <fstream>
#include <string.h>
#include <cmath>
#include "constants.h"
using namespace std;

#ifndef ORC_SEED
#define ORC_SEED 1
#endif
#ifndef ORC_NX
#define ORC_NX 65
#endif
#ifndef ORC_NINJECT
#define ORC_NINJECT 0
#endif
#ifndef ORC_TORR
#define ORC_TORR 0.2
#endif
#ifndef ORC_TEMPERATURE
#define ORC_TEMPERATURE 1.5
#endif
#ifndef ORC_ION_AMU
#define ORC_ION_AMU 39.948
#endif
#ifndef ORC_THRESHOLD
#define ORC_THRESHOLD 15.75
#endif
#ifndef ORC_COLLISIONS
#define ORC_COLLISIONS false
#endif
#ifndef ORC_SPECIES
#define ORC_SPECIES "ARGON"
#endif
#ifndef ORC_SIGMA_MODE
#define ORC_SIGMA_MODE "CONSTANT"
#endif
#ifndef ORC_SIGMA_CONST
#define ORC_SIGMA_CONST 0.0
#endif
#ifndef ORC_E_SEE
#define ORC_E_SEE "NO"
#endif
#ifndef ORC_I_SEE
#define ORC_I_SEE "NO"
#endif
#ifndef ORC_REFLECT
#define ORC_REFLECT "NO"
#endif
#ifndef ORC_BACKSCATTER
#define ORC_BACKSCATTER "NO"
#endif
#ifndef ORC_STEADY
#define ORC_STEADY "NO"
#endif
#ifndef ORC_DT_SCALE
#define ORC_DT_SCALE 0.1
#endif
#ifndef ORC_DTI_RATIO
#define ORC_DTI_RATIO 1.0
#endif
#ifndef ORC_BFIELD
#define ORC_BFIELD 0.0
#endif
#ifndef ORC_ANGLE_DEG
#define ORC_ANGLE_DEG 30.0
#endif
#ifndef ORC_PHI_LEFT
#define ORC_PHI_LEFT 0.0
#endif
#ifndef ORC_PHI_RIGHT
#define ORC_PHI_RIGHT 0.0
#endif
#ifndef ORC_PHI_PERIOD
#define ORC_PHI_PERIOD 0.0
#endif
#ifndef ORC_PHI_TOP
#define ORC_PHI_TOP 0.0
#endif
#ifndef ORC_PHI_BOTTOM
#define ORC_PHI_BOTTOM 0.0
#endif
#ifndef ORC_SIZE_TO_CHECK
#define ORC_SIZE_TO_CHECK 1000001
#endif

#define RAND_SEED ORC_SEED
#define INTERACTIVE "NO"
#define RESTART true
#define INIT_NO_NEUTRALS 10000
#define NUMBER_TO_INJECT ORC_NINJECT
#define ELECTRON_PARTICLE_DENSITY (double)1.0e15
#define ION_PARTICLE_DENSITY (double)1.0e15
#define GAS_PRESSURE ((double)ORC_TORR)*((double)133.32)
#define NEUTRAL_DENSITY (GAS_PRESSURE/((double)0.025*CHARGE))
#define TEMPERATURE (double)ORC_TEMPERATURE
#define VTE sqrt(TEMPERATURE*CHARGE/ELECTRON_MASS)
#define ION_MASS ((double)ORC_ION_AMU*AMU)
#define ION_CHARGE CHARGE
#define VTI sqrt(TEMPERATURE*CHARGE/ION_MASS)
#define VTN sqrt((double)0.025*CHARGE/ION_MASS)
#define THRESHOLD (double)ORC_THRESHOLD
#define WORK_FUNCTION (double)4.6
#define HAVE_COLLISIONS ORC_COLLISIONS
#define SPECIES ORC_SPECIES
#define SIGMA ORC_SIGMA_MODE
#define SIGMA_VALUE ORC_SIGMA_CONST
#define SIGMA_ELASTIC ORC_SIGMA_MODE
#define ELASTIC_SIGMA_VALUE ORC_SIGMA_CONST
#define SIGMA_IONIZATION ORC_SIGMA_MODE
#define IONIZATION_SIGMA_VALUE ORC_SIGMA_CONST
#define E_IMPACT_SEE ORC_E_SEE
#define ION_IMPACT_SEE ORC_I_SEE
#define REFLECTION ORC_REFLECT
#define BACKSCATTER ORC_BACKSCATTER
#define STEADYSTATE ORC_STEADY
#define X_NO_OF_CELLS ORC_NX
#define Y_NO_OF_CELLS ORC_NX
#define NO_OF_CELLS X_NO_OF_CELLS
#define NO_OF_DEBYE_LENGTHS (int)64
#define DEBYE_LENGTH sqrt((EPSILON*TEMPERATURE)/(ELECTRON_PARTICLE_DENSITY*CHARGE))
#define XLENGTH ((double)NO_OF_DEBYE_LENGTHS*DEBYE_LENGTH)
#define YLENGTH XLENGTH
#define LENGTH XLENGTH
#define DX (XLENGTH/(double)(X_NO_OF_CELLS-1))
#define DY (YLENGTH/(double)(Y_NO_OF_CELLS-1))
#define INIT_PARTICLE_NO 512*512
#define E_MACROPARTICLE_SIZE 1.0e6
#define ION_MACROPARTICLE_SIZE 1.0e6
#define PLASMA_FREQUENCY sqrt((ELECTRON_PARTICLE_DENSITY*ELECTRON_CHARGE2)/(EPSILON*ELECTRON_MASS))
#define DT ((double)ORC_DT_SCALE/PLASMA_FREQUENCY)
#define DTI ((double)ORC_DTI_RATIO*DT)
#define DT_DTI (int)(DTI/DT)
#define POTENTIAL_FREQUENCY (double)13.6e6
#define TWO_PI_F_DT (2.0*DT*PI*POTENTIAL_FREQUENCY)
#define PERIOD (1.0/TWO_PI_F_DT)
#define NO_GRAPH_STEPS ((int)50*(int)PERIOD)
#define TOTAL_RUN_TIME ((int)300*(int)PERIOD + 5)
#define START_GRAPH_TIME ((int)250*(int)PERIOD)
#define END_GRAPH_TIME (START_GRAPH_TIME+NO_GRAPH_STEPS)
#define TIME_DATA_FREQUENCY (int)100
#define SIZE_TIME_DATA TOTAL_RUN_TIME/TIME_DATA_FREQUENCY +(int)1
#define DXYPE XLENGTH/(sqrt(INIT_PARTICLE_NO) + 1.0)
#define DXYPI YLENGTH/(sqrt(INIT_PARTICLE_NO) + 1.0)
#define DXPE DXYPE
#define DXPI DXYPI
#define DYPE DXYPE
#define DYPI DXYPI
#define QCI (ION_MACROPARTICLE_SIZE*ION_CHARGE)
#define QCE (E_MACROPARTICLE_SIZE*ELECTRON_CHARGE)
#define Q_OVER_ME (ELECTRON_CHARGE/ELECTRON_MASS)
#define Q_OVER_MI (ION_CHARGE/ION_MASS)
#define MAGNETIC_FIELD (double)ORC_BFIELD
#define ANGLE ((double)ORC_ANGLE_DEG)*PI/((double)180.0)
#define PHI_LEFT (double)ORC_PHI_LEFT
#define PHI_RIGHT (double)ORC_PHI_RIGHT
#define PHI_PERIOD (double)ORC_PHI_PERIOD
#define PHI_TOP (double)ORC_PHI_TOP
#define PHI_BOTTOM (double)ORC_PHI_BOTTOM
#define NO_ION_SPECIES (int)1
#define NO_BINS 30001
#define DIVIDE_BINS_BY ((NO_BINS-1)/((int)100))
#define DIST_LOCATIONX (int)(0.9*(float)X_NO_OF_CELLS)
#define DIST_LOCATIONY (int)(0.5*(float)Y_NO_OF_CELLS)
#define DIST_LOCATION2X (int)(0.1*(float)X_NO_OF_CELLS)
#define DIST_LOCATION2Y (int)(0.5*(float)Y_NO_OF_CELLS)
#define SPREAD (int)(0.05*(float)X_NO_OF_CELLS)
#define POINT1X (int)3
#define POINT1Y (int)(Y_NO_OF_CELLS/2)
#define POINT2X (int)(X_NO_OF_CELLS/2)
#define POINT2Y (int)(Y_NO_OF_CELLS/2)
#define POINT3X (int)(X_NO_OF_CELLS -3)
#define POINT3Y (int)(Y_NO_OF_CELLS/2)
#define NO_TYPE (char *)"n"
#define ION_TYPE (char *)"i1"
#define ELECTRON_TYPE (char *)"e"
#define NO_GROUPS (int)3
#ifndef ORC_GROUP_LIMIT
#define ORC_GROUP_LIMIT 400000
#endif
#ifndef ORC_GROUP_LIMIT2
#define ORC_GROUP_LIMIT2 100000
#endif
#ifndef ORC_NEW_GROUP
#define ORC_NEW_GROUP 200000
#endif
#ifndef ORC_NEW_GROUP2
#define ORC_NEW_GROUP2 50000
#endif
#define UPPER_GROUP_LIMIT (int)ORC_GROUP_LIMIT
#define UPPER_GROUP_LIMIT2 (int)ORC_GROUP_LIMIT2
#define NEW_GROUP_SIZE (int)ORC_NEW_GROUP
#define NEW_GROUP_SIZE2 (int)ORC_NEW_GROUP2
#define UPPER_V_LIMIT ((double)1000.0*VTE)
#define UPPER_V_LIMIT_I ((double)1000.0*VTI)
#define VI1 (double)2.0*VTI
#define VI2 (double)3.0*VTI
#define VE1 (double)2.0*VTE
#define VE2 (double)3.0*VTE
#define SIZE_TO_CHECK (int)ORC_SIZE_TO_CHECK
#define SIZE_TO_CHECK_E (int)ORC_SIZE_TO_CHECK

#endif
