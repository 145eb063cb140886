/* Empty build configuration for compiling the reference headers in the
 * oracle harness: no MPI, Boost, NetCDF, ADOL-C or CUDA (every SCAFES_HAVE_*
 * switch stays undefined). */
#ifndef SCAFES_CONFIG_HPP_ORACLE_STUB
#define SCAFES_CONFIG_HPP_ORACLE_STUB
#endif
