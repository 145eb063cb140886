// Umbrella header of the GB300 drop-in for ScaFES (reference: src/ScaFES.hpp).
//
// A user problem written for ScaFES compiles unchanged against this
// directory (-I masterthesis_gb300/scafes -I include) and links
// libscafes_gb300.so; Problem::iterateOverTime then runs the update sweeps
// on the GPU.
#ifndef SCAFES_GB300_SCAFES_HPP
#define SCAFES_GB300_SCAFES_HPP

#include "ScaFES_Ntuple.hpp"
#include "ScaFES_Parameters.hpp"
#include "ScaFES_Grid.hpp"
#include "ScaFES_Sym.hpp"
#include "ScaFES_DataField.hpp"
#include "ScaFES_Problem.hpp"

#endif
