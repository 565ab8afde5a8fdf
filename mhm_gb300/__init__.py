"""mHM's water-balance step, parameter regionalisation and mRM routing on a
GB300, behind the C ABI of include/mhm_gpu.h (libmhm_gpu.so, built in-tree
by mhm_gb300.build).

Modules:
  model      MhmGpu (one basin, optionally many parameter sets as members)
             and MhmBatch (the fused multi-context launch)
  serve      the continuous-batching serving loop and the uneven-basins rounds
  network    the L11 network start-up from L0 flow data (host C++)
  routing    the link celerity of adaptive routing case 3 (L11_calc_celerity)
  restart    mHM / mRM restart files in the reference's layout
  outputs    aggregated flux/state outputs and the daily discharge file
  namelist   mhm.nml / mhm_parameter.nml reader and the run configuration
  params     global parameter vectors (gamma) of the process cases
  synth      seeded synthetic basins, level-0 maps and forcing
  h5read     the netCDF-4 / HDF5 reader used for the reference's files
"""
