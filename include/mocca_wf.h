/*
 * mocca_wf.h -- MOCCa wavefunction files (.wf, format version 1) for
 * libmocca_gpu.
 *
 * A file is the record sequence of WriteMOCCa_v1 / ReadMOCCa_v1
 * (src/InOut.f90:905-1416) as Fortran unformatted sequential records in
 * gfortran's layout: each record is a 4-byte little-endian byte count, the
 * payload and the count again; a payload above 2^31 - 9 bytes is split into
 * subrecords whose leading marker (all but the last) and trailing marker
 * (all but the first) carry the count negated.  Default INTEGER and LOGICAL
 * are 4 bytes (LOGICAL true = 1), REAL(dp) 8, COMPLEX(dp) 16 (re, im).
 *
 * Record order (one line per WRITE statement):
 *    1  version (= 1)
 *    2  TotalEnergy, TotalEnergy - OldEnergy
 *    3  nx, ny, nz, dx
 *    4  TRC, PC, SC, TSC, IC                               (logicals)
 *    5  nwt, neutrons, protons                             (int, 2 reals)
 *       per spwf (src/Spwf.f90:2246-2261):
 *         Grid(nx,ny,nz,4)
 *         Occupation, Energy, Dispersion, Norm, J(3),
 *         Isospin, TimeSimplex, Parity, Signature, TimeReversal
 *       densities (WriteDensity, src/Densities.f90:1189-1240):
 *         Rho(.,2), DerRho(.,3,2), LapRho(.,2) | Tau(.,2) | NablaJ(.,2) |
 *         JMuNu(.,3,3,2) or empty | five time-odd records or empty
 *    6  MaxFDOrder, MaxFDLapOrder, CoulombLapOrder
 *    7  afor                                               (character*200)
 *    8  t0,x0,t1,x1,t2,x2,t3a,x3a,yt3a,t3b,x3b,yt3b,wso,wsoq
 *    9  afor, hbar, hbm(2), COM1Body, COM2Body
 *   10  B1 ... B21 (28 reals)
 *   11  PairingType, PairingStrength(2), alpha(2), PairingCut(2)
 *   12  Pcutoffs(nwt) or empty
 *   13  Fermi(2), LNLambda(2)
 *   14  blocksizes(Pindex, Iindex)
 *   15  U, V                         (complex, HFBSize x 2 HFBSize x 2 x 2 each)
 *   16  HFBColumns(HFBSize, Pindex, Iindex)
 *   17  RhoHFB, KappaHFB             (complex, HFBSize x HFBSize x 2 x 2 each)
 *   18  CanTransfo                   (complex, HFBSize x HFBSize x blocks)
 *   19  Omega(3), CrankValues(3)
 *       per constrained moment (WriteMoment, src/Moments.f90:3330-3363):
 *         ConstraintType, Isoswitch, l, m, Impart
 *         Intensity(2), Constraint(2), TrueConstraint(2), Value(2), OldValue(2,7)
 *
 * Arrays keep the Fortran (column-major) element order, which is the
 * C-order of the reversed shape: a spwf grid is [4][nz][ny][nx], DerRho is
 * [2][3][nz][ny][nx], U is [2][2][2 HFBSize][HFBSize] complex.
 *
 * Status codes are those of mocca_gpu.h, plus MG_ERR_IO.
 */
#ifndef MOCCA_WF_H
#define MOCCA_WF_H

#include "mocca_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MG_ERR_IO  -6   /* file missing or unreadable, not version 1, or a record too short */

typedef struct mg_wf mg_wf;   /* one file's content, held in host memory */

/* Scalars of a file and the shapes of its arrays. */
typedef struct mg_wf_header {
    int    version;             /* 1                                                  */
    double energy, denergy;     /* TotalEnergy, TotalEnergy - OldEnergy (MeV)         */
    int    nx, ny, nz;          /* stored mesh points                                 */
    double dx;                  /* fm                                                 */
    int    trc, pc, sc, tsc, ic;/* conserved symmetries                               */
    int    nwt;                 /* stored spwfs                                       */
    double neutrons, protons;
    int    fd_order, fd_lap_order, coulomb_lap_order;   /* MaxFDOrder, MaxFDLapOrder,   */
                                                        /* CoulombLapOrder              */
    char   force[208];          /* afor without its blank padding, NUL-terminated     */
    double skyrme[14];          /* t0 x0 t1 x1 t2 x2 t3a x3a yt3a t3b x3b yt3b wso wsoq */
    double hbar, hbm[2];
    int    com1body, com2body;
    double coef[28];            /* B1 B2 B3 B4 B5 B6 B7a B7b B8a B8b Byt3a Byt3b B9 B9q */
                                /* B10 B11 B12a B12b B13a B13b B14 ... B21             */
    int    pairing_type;        /* 0 HF, 1 BCS, 2 HFB                                 */
    double pairing_strength[2], pairing_alpha[2], pairing_cut[2];
    double fermi[2], ln_lambda[2];
    double omega[3], crank_values[3];
    /* shapes: derived from the scalars above except where noted */
    int    hfb_size;            /* HFBSize: 2 nwt with time reversal, else nwt        */
    int    pindex, iindex;      /* 2 with parity / isospin conserved, else 1          */
    int    can_blocks;          /* (P, it) blocks of CanTransfo on file (as read)     */
    int    has_cutoffs;         /* record 12 holds Pcutoffs(nwt)                      */
    int    has_jmunu;           /* the JMuNu record is not empty                      */
    int    odd_records;         /* bit k: time-odd density record k+1 is not empty    */
    int    n_moments;           /* constrained moments at the end                     */
} mg_wf_header;

/* Array fields of a file (mg_wf_field); element type and count per field: */
#define MG_WF_GRIDS        0   /* double nwt*4V                                   */
#define MG_WF_SPWF_REAL    1   /* double nwt*7: occupation energy dispersion norm J(3) */
#define MG_WF_SPWF_INT     2   /* int nwt*5: isospin timesimplex parity signature  */
                               /*            timereversal                          */
#define MG_WF_RHO          3   /* double 2V                                        */
#define MG_WF_DERRHO       4   /* double 6V                                        */
#define MG_WF_LAPRHO       5   /* double 2V                                        */
#define MG_WF_TAU          6   /* double 2V                                        */
#define MG_WF_NABLAJ       7   /* double 2V                                        */
#define MG_WF_JMUNU        8   /* double 18V or 0                                  */
#define MG_WF_ODD1         9   /* double 12V or 0: vecj(.,3,2), rotvecj(.,3,2)     */
#define MG_WF_ODD2        10   /* double 30V or 0: vecs, rots, ders(.,3,3,2)       */
#define MG_WF_ODD3        11   /* double 14V or 0: laps(.,3,2), divs(.,2),         */
                               /*                  graddivs(.,3,2)                 */
#define MG_WF_ODD4        12   /* double 6V or 0: vecT                             */
#define MG_WF_ODD5        13   /* double 6V or 0: vecF                             */
#define MG_WF_CUTOFFS     14   /* double nwt or 0                                  */
#define MG_WF_BLOCKSIZES  15   /* int pindex*iindex                                */
#define MG_WF_U           16   /* double 2*hfb*2hfb*4 (complex as re, im)          */
#define MG_WF_V           17   /* double 2*hfb*2hfb*4                              */
#define MG_WF_COLUMNS     18   /* int hfb*pindex*iindex                            */
#define MG_WF_RHOHFB      19   /* double 2*hfb*hfb*4                               */
#define MG_WF_KAPPAHFB    20   /* double 2*hfb*hfb*4                               */
#define MG_WF_CANTRANSFO  21   /* double 2*hfb*hfb*can_blocks                      */
#define MG_WF_MOMENT_INT  22   /* int n_moments*5: type isoswitch l m impart       */
#define MG_WF_MOMENT_REAL 23   /* double n_moments*22: intensity(2) constraint(2)  */
                               /*   trueconstraint(2) value(2) oldvalue(2,7)       */
#define MG_WF_NFIELDS     24

/* ---- the file object (host only, no device work) ---------------------- */

/* Parse a file as ReadMOCCa_v1 does (src/InOut.f90:1050-1416): every record
 * in order, the version must be 1, every spwf's isospin +-1 (ReadSpwf,
 * src/Spwf.f90:2283-2285).  A record shorter than the items read from it is
 * an error; a longer one is accepted with its tail ignored, as a Fortran
 * READ does.  Moment records run to the end of the file. */
int mg_wf_load(const char* path, mg_wf** out);
/* An empty file object with the header's scalars and shapes (hfb_size,
 * pindex, iindex follow from nwt and the symmetries; can_blocks 0 means
 * pindex * iindex); every array zero. */
int mg_wf_new(const mg_wf_header* h, mg_wf** out);
/* Write the records in WriteMOCCa_v1's order (src/InOut.f90:963-1046). */
int mg_wf_save(const mg_wf* wf, const char* path);
int mg_wf_free(mg_wf* wf);
int mg_wf_get_header(const mg_wf* wf, mg_wf_header* out);
/* Replace the scalars (energy ... crank_values); the shapes stay. */
int mg_wf_set_scalars(mg_wf* wf, const mg_wf_header* h);
/* Pointer to a field's elements (writable) and their count (doubles or
 * ints, see the table above); a field absent from the file has count 0. */
int mg_wf_field(mg_wf* wf, int field, void** data, long long* count);

/* ---- a device context and a file --------------------------------------- */

/* The context's state as WriteMOCCa_v1 writes it: HF spwfs with their
 * occupations, energies, dispersions, norms <psi|psi> and <J> (DiagAng,
 * src/Spwf.f90:976-1085), the densities (with time reversal broken the
 * current and spin densities and their curls; records the context does
 * not hold are written empty, which ReadDensity reads as zero), the force
 * and its B-coefficients, the pairing parameters, cutoffs and Fermi
 * energies, and the HFB matrices of the last pairing step: U and V from
 * its quasiparticle vectors (DiagonaliseHFBHamiltonian_Signature,
 * src/HFB.f90:2695-2786) with HFBColumns as src/HFB.f90:1008-1019 chooses
 * them, the mixed RhoHFB and KappaHFB, and CanTransfo in DiagonaliseRhoHFB's
 * column order (src/HFB.f90:3156-3284).  An HF context writes the guess
 * of GuessHFBMatrices(0) (src/HFB.f90:3645-3718) instead.  force_name may
 * be NULL; the constrained moments are written with their current values. */
int mg_wf_from_context(mg_ctx* ctx, const char* force_name, mg_wf** out);
/* Restart a context from a file (ReadMOCCa_v1 and Input, src/InOut.f90:
 * 123-192, with the file's mesh, symmetries and nwt equal to the
 * context's): HF spwfs with quantum numbers, occupations and energies;
 * the densities; under HFB the Fermi energies and RhoHFB / KappaHFB, which
 * the next pairing step starts from (TransformHFBMatrices,
 * src/Transform.f90:1056-1064), with no mixing history.  The force and
 * pairing parameters stay those of the context, as the reference keeps its
 * input data's. */
int mg_wf_to_context(mg_ctx* ctx, const mg_wf* wf);

/* DiagAng's <J> (src/Spwf.f90:976-1085) of every spwf of a basis:
 * out[3*i + 0..2] = <Jx>, <Jy>, <Jz> (components a conserved signature or
 * time simplex makes zero are zero).  Derives the basis first. */
int mg_angular_momentum(mg_ctx* ctx, int basis, double* out);

#ifdef __cplusplus
}
#endif

#endif /* MOCCA_WF_H */
