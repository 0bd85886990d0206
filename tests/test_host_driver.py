"""The host side above the C ABI: parameters.h reader and text formats.

pgb_params_from_header evaluates a parameters.h the way the compiler does
(parameters.h:41-366 with constants.h), so the derived quantities of a run
come from the user's own file; these tests need no GPU.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO

PARAMS_TEXT = r'''
#ifndef parameters_h
#define parameters_h
#include "constants.h"
#define RAND_SEED time(NULL)
#define INTERACTIVE "NO" // "NO" // "YES"
#define RESTART true  //true // false
#define INIT_NO_NEUTRALS 10000
#define NUMBER_TO_INJECT 10
#define ELECTRON_PARTICLE_DENSITY (double)1.0e15
#define ION_PARTICLE_DENSITY (double)1.0e15
#define GAS_PRESSURE ((double)0.2)*((double)133.32) //Gas pressure in pascals.
#define NEUTRAL_DENSITY (GAS_PRESSURE/((double)0.025*CHARGE))
#define TEMPERATURE  (double)3.0
#define VTE sqrt(TEMPERATURE*CHARGE/ELECTRON_MASS)  // electron thermal velocity
#define ION_MASS ((double)AMU)               // mass of the ion
#define ION_CHARGE CHARGE
#define VTI sqrt(TEMPERATURE*CHARGE/ION_MASS)
#define VTN sqrt((double)0.025*CHARGE/ION_MASS)
#define THRESHOLD (double)13.6
#define WORK_FUNCTION (double)4.6
#define HAVE_COLLISIONS true  // true  // true if want collisions
#define SPECIES  "HYDROGEN" // "ARGON" // "HYDROGEN"
#define SIGMA "ENERGY_DEPENDENT"
#define SIGMA_VALUE 0.0
#define SIGMA_ELASTIC "ENERGY_DEPENDENT"
#define ELASTIC_SIGMA_VALUE 0.0 //double type
#define SIGMA_IONIZATION "ENERGY_DEPENDENT"
#define IONIZATION_SIGMA_VALUE 0.0 //double type
#define E_IMPACT_SEE "YES"  // "YES" // "NO"
#define ION_IMPACT_SEE "NO"
#define REFLECTION  "YES"
#define BACKSCATTER  "YES"
#define STEADYSTATE "NO" //  "NO" //"YES"
#define X_NO_OF_CELLS 129
#define Y_NO_OF_CELLS 129
#define NO_OF_CELLS X_NO_OF_CELLS
#define NO_OF_DEBYE_LENGTHS (int)64
#define DEBYE_LENGTH sqrt((EPSILON*TEMPERATURE)/(ELECTRON_PARTICLE_DENSITY*CHARGE))
#define XLENGTH ((double)NO_OF_DEBYE_LENGTHS*DEBYE_LENGTH)
#define YLENGTH XLENGTH
#define LENGTH XLENGTH
#define DX (XLENGTH/(double)(X_NO_OF_CELLS-1))
#define DY (YLENGTH/(double)(Y_NO_OF_CELLS-1))
#define INIT_PARTICLE_NO 64*64
#define E_MACROPARTICLE_SIZE 1.0e6
#define ION_MACROPARTICLE_SIZE 1.0e6
#define PLASMA_FREQUENCY sqrt((ELECTRON_PARTICLE_DENSITY*ELECTRON_CHARGE2)/(EPSILON*ELECTRON_MASS))
#define DT ((double)0.1/PLASMA_FREQUENCY)  //Electron time-step
#define DTI ((double)1.0*DT) //Ion time-step
#define DT_DTI (int)(DTI/DT) //Ratio of ion time-step over electron
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
#define DXPE  DXYPE
#define DXPI  DXYPI
#define DYPE  DXYPE
#define DYPI  DXYPI
#define QCI (ION_MACROPARTICLE_SIZE*ION_CHARGE)
#define QCE (E_MACROPARTICLE_SIZE*ELECTRON_CHARGE)
#define Q_OVER_ME (ELECTRON_CHARGE/ELECTRON_MASS)
#define Q_OVER_MI (ION_CHARGE/ION_MASS)
#define  MAGNETIC_FIELD (double)0.02
#define  ANGLE ((double)30.0)*PI/((double)180.0)
#define PHI_LEFT (double)0.0  // left boundary voltage
#define PHI_RIGHT (double)5.0
#define PHI_PERIOD (double)0.001   // voltage period
#define PHI_TOP (double)0.0  // voltage of top boundary
#define PHI_BOTTOM (double)-1.0  // voltage of bottom boundary
#define NO_ION_SPECIES (int)1
#define NO_BINS 30001  // number of velocity bins
#define DIVIDE_BINS_BY ((NO_BINS-1)/((int)100))  // used for scaling
#define DIST_LOCATIONX  (int)(0.9*(float)X_NO_OF_CELLS)
#define SPREAD (int)(0.05*(float)X_NO_OF_CELLS)
#define POINT1X  (int)3
#define POINT1Y  (int)(Y_NO_OF_CELLS/2)
#define POINT2X  (int)(X_NO_OF_CELLS/2)
#define POINT2Y  (int)(Y_NO_OF_CELLS/2)
#define POINT3X  (int)(X_NO_OF_CELLS -3)
#define POINT3Y  (int)(Y_NO_OF_CELLS/2)
#define NO_TYPE (char *)"n"  // no type
#define ION_TYPE (char *)"i1"  // ions
#define ELECTRON_TYPE (char *)"e"  // electrons
#define NO_GROUPS (int)3
#define UPPER_GROUP_LIMIT (int)400000
#define UPPER_GROUP_LIMIT2 (int)100000
#define NEW_GROUP_SIZE (int)200000
#define NEW_GROUP_SIZE2 (int)50000
#define UPPER_V_LIMIT ((double)1000.0*VTE)
#define UPPER_V_LIMIT_I ((double)1000.0*VTI)
#define VI1 (double)2.0*VTI
#define VI2 (double)3.0*VTI
#define VE1 (double)2.0*VTE
#define VE2 (double)3.0*VTE
#define SIZE_TO_CHECK (int)1000001
#define SIZE_TO_CHECK_E (int)1000001
#endif
'''


def test_parameters_h_reader_matches_make_params(lib, tmp_path):
    import picgb
    path = tmp_path / "parameters.h"
    path.write_text(PARAMS_TEXT)
    got = picgb.PgbParams()
    lib.pgb_params_from_header.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(picgb.PgbParams)]
    assert lib.pgb_params_from_header(str(path).encode(), 7, C.byref(got)) == 0
    want = picgb.make_params(X_NO_OF_CELLS=129, TEMPERATURE=3.0, ION_MASS_AMU=1.0, THRESHOLD=13.6,
                             HAVE_COLLISIONS=True, SPECIES="HYDROGEN", SIGMA="ENERGY_DEPENDENT",
                             SIGMA_ELASTIC="ENERGY_DEPENDENT", SIGMA_IONIZATION="ENERGY_DEPENDENT",
                             E_IMPACT_SEE="YES", REFLECTION="YES", BACKSCATTER="YES", STEADYSTATE="NO",
                             NUMBER_TO_INJECT=10, MAGNETIC_FIELD=0.02, PHI_RIGHT=5.0, PHI_PERIOD=0.001,
                             PHI_BOTTOM=-1.0, RAND_SEED=7)
    for name, _ in picgb.PgbParams._fields_:
        a, b = getattr(got, name), getattr(want, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name


def test_parameters_h_reader_rejects_missing_file(lib):
    import picgb
    got = picgb.PgbParams()
    lib.pgb_params_from_header.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(picgb.PgbParams)]
    assert lib.pgb_params_from_header(b"/nonexistent/parameters.h", 1, C.byref(got)) == -6


def _reference_dir():
    """The reference's source directory that oracle/Makefile built oracle/_ref
    from (recorded there), or None where it was not built."""
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "refdir")
    try:
        d = open(path).read().strip()
    except OSError:
        return None
    return d if os.path.isdir(d) else None


@pytest.mark.skipif(_reference_dir() is None, reason="reference presets not present")
def test_reference_presets_parse(lib):
    import picgb
    lib.pgb_params_from_header.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(picgb.PgbParams)]
    for d, species, steady in (("", 0, 1), ("parameter file for Ar steadystate", 0, 1),
                               ("parameter file for Ar with coll-boundary", 0, 0),
                               ("parameter file for H with coll-boundary", 1, 0)):
        got = picgb.PgbParams()
        path = os.path.join(_reference_dir(), d, "parameters.h")
        assert lib.pgb_params_from_header(path.encode(), 1, C.byref(got)) == 0, path
        assert got.x_no_of_cells == 257 and got.species == species and got.steadystate == steady
