# libsaisConfig.cmake -- find_package(libsais CONFIG) for libsais_gb300.
#
# Provides the imported target `libsais`, the name the reference exports from
# its own build (CMakeLists.txt: add_library(libsais), install(EXPORT
# libsaisTargets FILE libsaisConfig.cmake)), so an application that does
#
#     find_package(libsais CONFIG REQUIRED)
#     target_link_libraries(app PRIVATE libsais)
#
# links the GPU build instead without changing its own CMake code.  The
# target's include directory holds libsais.h, libsais64.h, libsais16.h,
# libsais16x64.h (the reference's declarations) and libsais_gb300.h (the GPU
# extensions); the library is libsais_gb300/lib/libsais_gb300.so, built by
# `python -c "import __graft_entry__ as g; g.build()"`.
get_filename_component(_libsais_gb300_root "${CMAKE_CURRENT_LIST_DIR}/../.." ABSOLUTE)
set(_libsais_gb300_so "${_libsais_gb300_root}/libsais_gb300/lib/libsais_gb300.so")
if(NOT EXISTS "${_libsais_gb300_so}")
    set(libsais_FOUND FALSE)
    set(libsais_NOT_FOUND_MESSAGE "libsais_gb300 is not built: ${_libsais_gb300_so} is missing")
    return()
endif()
if(NOT TARGET libsais)
    add_library(libsais SHARED IMPORTED)
    set_target_properties(libsais PROPERTIES
        IMPORTED_LOCATION "${_libsais_gb300_so}"
        IMPORTED_NO_SONAME TRUE
        INTERFACE_INCLUDE_DIRECTORIES "${_libsais_gb300_root}/include")
endif()
set(libsais_INCLUDE_DIR "${_libsais_gb300_root}/include")
set(libsais_LIBRARY "${_libsais_gb300_so}")
unset(_libsais_gb300_root)
unset(_libsais_gb300_so)
