/* Empty stand-in for the Win32 header that the reference's sources include
 * unconditionally (particle.h, pic.h, openCLutility.h).  Nothing from it is
 * used on the simulation path.  Test infrastructure only. */
#pragma once
