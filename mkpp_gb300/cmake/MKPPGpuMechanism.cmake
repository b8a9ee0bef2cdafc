# CMake entry point for host models that link the GPU mechanism libraries.
#
# The counterpart of the reference's mkpp_add_compiled_mechanism
# (src/mkpp_host/cmake/MKPPCompiledMechanism.cmake:9-53).  There, a generated
# mechanism's C++ sources become a static library that links Kokkos.  Here a
# mechanism is one shared library, libmkpp_<mechanism>.so, that mkpp_gb300's
# build step compiles with nvcc for sm_103a.  CMake runs that step at build
# time, and the step rebuilds only what is stale.  The consumer gets the
# library and the include directory of its mkpp.h, the per-mechanism header
# with the C ABI and MKPP_NUM_* sizes.
#
#   include(<mkpp_gb300>/cmake/MKPPGpuMechanism.cmake)
#   mkpp_gpu_add_mechanism(chem_saprc99 saprc99)
#   target_link_libraries(host_model PRIVATE chem_saprc99)
#
#   # the header-only MechanismRegistry (mkpp_host/mechanism_manager.hpp),
#   # which finds mechanisms in the in-tree library directory at run time
#   target_link_libraries(host_model PRIVATE mkpp_gb300::registry)
#
# Only one mechanism library may be linked into one program: the C ABI's
# symbols are not namespaced by mechanism, as in the reference.  A program that
# needs several mechanisms goes through mkpp_gb300::registry, which loads each
# library on its own.
include_guard(GLOBAL)

get_filename_component(MKPP_GB300_PACKAGE_DIR "${CMAKE_CURRENT_LIST_DIR}/.." ABSOLUTE)
get_filename_component(MKPP_GB300_ROOT "${MKPP_GB300_PACKAGE_DIR}/.." ABSOLUTE)
set(MKPP_GB300_LIB_DIR "${MKPP_GB300_PACKAGE_DIR}/lib")

find_package(Python3 REQUIRED COMPONENTS Interpreter)

if(NOT TARGET mkpp_gb300::registry)
  add_library(mkpp_gb300_registry INTERFACE)
  target_include_directories(mkpp_gb300_registry INTERFACE "${MKPP_GB300_ROOT}/include")
  target_compile_definitions(mkpp_gb300_registry INTERFACE "MKPP_GB300_LIB_DIR=\"${MKPP_GB300_LIB_DIR}\"")
  target_compile_features(mkpp_gb300_registry INTERFACE cxx_std_17)
  target_link_libraries(mkpp_gb300_registry INTERFACE ${CMAKE_DL_LIBS})
  # Header-only NVTX3 from the CUDA toolkit: the batched dispatch's profiler range.
  find_package(CUDAToolkit QUIET)
  if(TARGET CUDA::nvtx3)
    target_link_libraries(mkpp_gb300_registry INTERFACE CUDA::nvtx3)
  endif()
  add_library(mkpp_gb300::registry ALIAS mkpp_gb300_registry)
endif()

# mkpp_gpu_add_mechanism(<target> <mechanism>)
#
# <target> is an INTERFACE library carrying libmkpp_<mechanism>.so and the
# include directory of its mkpp.h.  A mechanism without a plan under
# mkpp_gb300/mechanisms/ is an error at configure time, as the reference's
# function stops on a mechanism without generated sources.
function(mkpp_gpu_add_mechanism target mechanism)
  set(plan "${MKPP_GB300_PACKAGE_DIR}/mechanisms/${mechanism}.plan.json")
  if(NOT EXISTS "${plan}")
    message(FATAL_ERROR "FATAL ERROR: ${mechanism} has no plan in ${MKPP_GB300_PACKAGE_DIR}/mechanisms")
  endif()
  set(lib "${MKPP_GB300_LIB_DIR}/libmkpp_${mechanism}.so")
  # The build step decides staleness itself (sources newer than the
  # library), so it runs on every build and is a no-op when nothing changed.
  add_custom_target(${target}_build
    COMMAND "${Python3_EXECUTABLE}" -m mkpp_gb300.build "${mechanism}"
    WORKING_DIRECTORY "${MKPP_GB300_ROOT}"
    BYPRODUCTS "${lib}"
    COMMENT "mkpp_gb300: libmkpp_${mechanism}.so (sm_103a)"
    VERBATIM)
  add_library(${target} INTERFACE)
  target_include_directories(${target} INTERFACE "${MKPP_GB300_PACKAGE_DIR}/generated/host_api/${mechanism}")
  target_link_libraries(${target} INTERFACE "${lib}")
  add_dependencies(${target} ${target}_build)
endfunction()
