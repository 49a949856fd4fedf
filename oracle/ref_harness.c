/*
 * ref_harness.c -- glue that lets the reference's own KLM exact-diagonalisation objects
 * (main/exact_diag/klm_vf/src/{FIND_DIM,GET_BASIS,GET_HAM,MAKE_ELEMENT_HAM}.c) link into
 * oracle/_ref.
 *
 * TEST INFRASTRUCTURE ONLY.  The driver's GET_HAM_BOX.c / FREE_HAM_BOX.c do not compile as
 * shipped (they use MODEL_1DKLM_VF fields that include/model.h does not define), so this
 * file supplies both with the operator set MAKE_ELEMENT_HAM reads
 * (main/exact_diag/klm_vf/src/GET_HAM_BOX.c:18-34), built by the reference's own
 * onsite_op routines.  The observable / SC-correlation operators are not needed here.
 */
#include <stdlib.h>

#include "Header.h"

HAM_BOX *GET_HAM_BOX(MODEL_1DKLM_VF *Model) {
   const int d = Model->dim_onsite, s = Model->spin_loc;
   HAM_BOX *Box = calloc(1, sizeof(*Box));
   Box->Ham_On = GET_CRS1(d, d * d);
   Box->SpL_On = GET_CRS1(d, d * d);
   Box->SmL_On = GET_CRS1(d, d * d);
   Box->SzL_On = GET_CRS1(d, d * d);
   Box->CUp_On = GET_CRS1(d, d * d);
   Box->CUp_D_On = GET_CRS1(d, d * d);
   Box->CDown_On = GET_CRS1(d, d * d);
   Box->CDown_D_On = GET_CRS1(d, d * d);
   Box->Zero_On = GET_CRS1(d, d * d);
   ONSITE_MAKE_HAM_SZBASIS_KLM(Model, Box->Ham_On);
   ONSITE_SPL_SZBASIS_KLM(s, Box->SpL_On, 1.0);
   ONSITE_SML_SZBASIS_KLM(s, Box->SmL_On, 1.0);
   ONSITE_SZL_SZBASIS_KLM(s, Box->SzL_On, 1.0);
   ONSITE_CUP_SZBASIS_KLM(s, Box->CUp_On, 1.0);
   ONSITE_CUP_DAGGER_SZBASIS_KLM(s, Box->CUp_D_On, 1.0);
   ONSITE_CDOWN_SZBASIS_KLM(s, Box->CDown_On, 1.0);
   ONSITE_CDOWN_DAGGER_SZBASIS_KLM(s, Box->CDown_D_On, 1.0);
   ONSITE_DIAG_SZBASIS_KLM(s, Box->Zero_On, 0.0);
   return Box;
}

void FREE_HAM_BOX(HAM_BOX *Box, MODEL_1DKLM_VF *Model) {
   (void)Model;
   FREE_CRS1(Box->Ham_On);
   FREE_CRS1(Box->SpL_On);
   FREE_CRS1(Box->SmL_On);
   FREE_CRS1(Box->SzL_On);
   FREE_CRS1(Box->CUp_On);
   FREE_CRS1(Box->CUp_D_On);
   FREE_CRS1(Box->CDown_On);
   FREE_CRS1(Box->CDown_D_On);
   FREE_CRS1(Box->Zero_On);
   free(Box);
}

/* Site operator tables of the KLM basis, for comparing the restated tables against the
 * reference's: which = 0 Ham_On, 1 SpL, 2 SmL, 3 SzL, 4 CUp, 5 CUp_D, 6 CDown, 7 CDown_D, 8 Zero. */
int ref_klm_site_op(MODEL_1DKLM_VF *Model, int which, long *row, int *col, double *val) {
   HAM_BOX *B = GET_HAM_BOX(Model);
   CRS1 *tab[9] = {B->Ham_On, B->SpL_On, B->SmL_On, B->SzL_On, B->CUp_On, B->CUp_D_On, B->CDown_On, B->CDown_D_On, B->Zero_On};
   if (which < 0 || which > 8) return -1;
   CRS1 *M = tab[which];
   const int d = Model->dim_onsite;
   for (int i = 0; i <= d; i++) row[i] = M->Row[i];
   for (long k = 0; k < M->Row[d]; k++) {
      col[k] = M->Col[k];
      val[k] = M->Val[k];
   }
   int nnz = (int)M->Row[d];
   FREE_HAM_BOX(B, Model);
   return nnz;
}
