// Test infrastructure only: the few symbols of the reference's Utils.cpp and
// flex/bison parser that IoData.cpp references, for the single-rank oracle
// build of the reference's EOS / flux / exact-Riemann sources.
#include <cstdio>
#include <cstdarg>
#include <cstdlib>
#include <ctime>
FILE* yyCmdfin = nullptr;
int yyCmdfparse() { return 0; }
void exit_mpi() { std::exit(-1); }
void print(const char* fmt, ...) { va_list a; va_start(a, fmt); vfprintf(stdout, fmt, a); va_end(a); }
void print(FILE* f, const char* fmt, ...) { va_list a; va_start(a, fmt); vfprintf(f, fmt, a); va_end(a); }
void print_error(const char* fmt, ...) { va_list a; va_start(a, fmt); vfprintf(stderr, fmt, a); va_end(a); }
double MPI_Wtime() { return (double)clock() / CLOCKS_PER_SEC; }
