/* Stand-in for HYPRE's utilities header -- TEST INFRASTRUCTURE ONLY (see HYPRE_struct_ls.h). */
#ifndef IMPEC_REFSHIM_HYPRE_UTILITIES_H
#define IMPEC_REFSHIM_HYPRE_UTILITIES_H
typedef int HYPRE_Int;
typedef double HYPRE_Real;
#endif
