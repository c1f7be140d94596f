/* design_oracle.h -- CPU restatement of the design-update chain (density
 * filter, tanh projection, MMA) used only as the oracle of the GPU design
 * update.  Test infrastructure. */
#ifndef LBM_DESIGN_ORACLE_H
#define LBM_DESIGN_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* One filter stage: cone density filter of radius `radius` on the cells of
 * `box` (identity elsewhere), then, if `project`, the tanh projection. */
typedef struct dsg_stage {
  int radius;
  int box[6];
  int project;
  double beta, eta;
} dsg_stage;

typedef struct dsg_chain {
  int nx, ny, nz;
  int nstages;
  dsg_stage stage[2];
} dsg_chain;

/* gamma = stages applied to the full-grid field xfull */
int dsg_filter_forward(const dsg_chain* ch, const double* xfull, double* gamma);
/* s (dJ/dgamma on entry) <- dJ/dxfull, the chain rule at xfull */
int dsg_filter_transpose(const dsg_chain* ch, const double* xfull, double* s);

typedef struct dsg_mma dsg_mma;
/* n variables, m constraints; a = the constants a_j of the constraints'
 * z terms (NULL: 0; 1 for the min-max form) */
dsg_mma* dsg_mma_create(int n, int m, const double* x0, const double* a);
void dsg_mma_destroy(dsg_mma* s);
/* x <- new design; df0: n, g: m, dg: m x n (row j = constraint j) */
int dsg_mma_update(dsg_mma* s, double* x, const double* df0, const double* g, const double* dg,
                   double movlim, int* dual_iterations, double* change);
const double* dsg_mma_lambda(const dsg_mma* s);

#ifdef __cplusplus
}
#endif

#endif
