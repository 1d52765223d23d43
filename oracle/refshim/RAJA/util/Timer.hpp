/* RAJA::Timer comes with the stand-in RAJA header (test infrastructure only). */
#include <RAJA/RAJA.hpp>
