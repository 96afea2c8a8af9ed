// Forwarding header of the project-written AMReX stand-in.
#include "mph_amrex_standin.H"
