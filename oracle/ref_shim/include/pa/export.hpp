// Shim for the CMake-generated export header of libpa (pa/CMakeLists.txt:92-98).
// The oracle build links the reference sources into one shared object with
// default visibility, so the export macro expands to nothing.
#ifndef PA_EXPORT_HPP
#define PA_EXPORT_HPP
#define PA_EXPORT
#endif
