/* Stand-in for the CMake-generated export header of the reference build:
   symbols are exported with default visibility. Test infrastructure only. */
#ifndef GIMLI_EXPORT_STANDIN_H
#define GIMLI_EXPORT_STANDIN_H
#define DLLEXPORT
#endif
