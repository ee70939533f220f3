/* PIHM input decks: the reference's text input files read and initialised on
 * the host, so that the same watershed on disk feeds this library, the
 * reference and its CPU restatement.
 *
 * A deck is <dir>/<proj>.{riv,mesh,att,soil,para,meteo,bc} (and .lai when
 * an element names an LAI series) with <dir>/<project>.calib (and
 * <dir>/<project>.ic for a hot start), where <proj> is <project> up to its
 * first '.', plus the land-cover table (the reference reads
 * input/vegprmt.tbl).  Reading follows ReadAlloc (src/read_alloc.c:3-162:
 * ReadRiver, ReadMesh, ReadAtt, ReadSoil, ReadLc, ReadForc, ReadLai,
 * ReadPara, ReadCalib, ReadBc) and initialisation follows Initialize
 * (src/initialize.c:9-222: InitMesh, InitTopo, InitSoil, InitLc, InitForc,
 * InitRiver, CorrElev when asked, InitSurfL, then RelaxIc or ReadIc).  Unlike the reference, a malformed deck returns
 * an error code with a message instead of exiting the process.
 *
 * Host only; nothing here touches the GPU. */
#ifndef PIHM_DECK_H
#define PIHM_DECK_H

#include <stdint.h>

#include "pihm_batch.h"
#include "pihm_gpu.h"
#include "pihm_land.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pihm_deck pihm_deck;

enum {
    PIHM_DECK_ERR_IO = -20,     /* a file of the deck cannot be opened */
    PIHM_DECK_ERR_FORMAT = -21, /* a line does not have the expected form */
    PIHM_DECK_ERR_VALUE = -22   /* a value is out of range (index, porosity, ...) */
};

/* Flags of pihm_deck_read. */
#define PIHM_DECK_CORR_ELEV 1   /* lift sink elements as CorrElev does (the reference's -c option) */

/* Read and initialise a deck.  lc_table: path of the land-cover table, or
 * NULL for <dir>/../vegprmt.tbl (the reference's input/vegprmt.tbl next to
 * input/<proj>/).  Returns 0 or a negative code; pihm_deck_error gives the
 * message of the last failure on the calling thread. */
int pihm_deck_read(const char *dir, const char *project, const char *lc_table, int flags,
                   pihm_deck **out);
const char *pihm_deck_error(void);
void pihm_deck_free(pihm_deck *deck);

/* The initialised watershed, reference order.  The pointers stay valid until
 * pihm_deck_free; pass the struct to pihm_gpu_create or a batch job. */
int pihm_deck_mesh(const pihm_deck *deck, pihm_gpu_mesh *mesh);

/* The model controls of the .para file (src/read_para.c:3-200). */
typedef struct pihm_deck_control {
    int32_t surf_mode, riv_mode, unsat_mode;
    int32_t init_mode;            /* 0 relaxation (RelaxIc), 1 restart file (.ic) */
    int64_t start, end;           /* simulation period, seconds since 1970-01-01 UTC */
    int32_t lsm_step;             /* land-surface (ET) step, s */
    pihm_step_control step;       /* model step, tolerances, AdjCVodeMaxStep factors */
} pihm_deck_control;
int pihm_deck_control_get(const pihm_deck *deck, pihm_deck_control *ctrl);

/* Initial state [3*nelem + 2*nriver] in reference order: RelaxIc
 * (src/initialize.c:496-575) or the .ic restart file (src/read_ic.c:3-39). */
int pihm_deck_initial_state(const pihm_deck *deck, double *y0);

/* Canopy storage and snow water equivalent at the start [nelem], for
 * pihm_gpu_land_set_state: 0 after RelaxIc (src/initialize.c:509-510), the
 * restart file's ic.cmc and ic.sneqv otherwise (src/read_ic.c:3-39,
 * src/initialize.c:594-595); either may be NULL. */
int pihm_deck_initial_storage(const pihm_deck *deck, double *cmc, double *sneqv);

/* The land-surface model of the deck for pihm_gpu_land_init: the element
 * parameters InitSoil, InitLc and InitForc leave (src/init_soil.c:34-54 with
 * FieldCapacity and WiltingPoint of the soil table, src/soil.c:16-81;
 * src/init_lc.c:19-38; the station's wind height, src/init_forc.c:81-85)
 * and the .meteo and .lai series (src/read_forc.c, src/read_lai.c) with the
 * calibration's climate scenario applied.  The pointers stay valid until
 * pihm_deck_free. */
int pihm_deck_land(const pihm_deck *deck, pihm_land_params *params, pihm_forcing_series *series);

/* Boundary values at time t (seconds since 1970-01-01 UTC) as ApplyBc sets
 * them (src/forcing.c:24-249): elem_bc [3*nelem] (element-major, edge j of
 * element i at 3*i + j: the head of a Dirichlet edge, the flux of a Neumann
 * edge, 0 elsewhere) and river_bc [nriver]; either may be NULL.  The
 * series are interpolated linearly as IntrplForc does (src/forcing.c:482-531);
 * a time outside a series returns PIHM_DECK_ERR_VALUE. */
int pihm_deck_bc(const pihm_deck *deck, int64_t t, double *elem_bc, double *river_bc);

#ifdef __cplusplus
}
#endif
#endif /* PIHM_DECK_H */
