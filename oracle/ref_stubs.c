/*
 * No-op definitions that let the reference's unmodified src/fluid.c and
 * src/hash.c link into a shared library for the test oracle (oracle/_ref).
 *
 * fluid.c references MPI (fluid.c:51-364), the render rank (fluid.c:63),
 * the domain decomposition (fluid.c:147-150, geometry.c) and the halo /
 * migration exchange (fluid.c:318-345, communication.c).  None of those are
 * on the compute path the oracle drives: the harness in ref_driver.c calls
 * the step functions (fluid.c:398-744, hash.c:35-242) directly on a single
 * domain, exactly as one compute rank with no neighbours would.
 *
 * Test infrastructure only: never linked into the product library.
 */
#include "fluid.h"

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; *r = MPI_REQUEST_NULL; return 0; }
int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)s; *r = MPI_REQUEST_NULL; return 0; }
int MPI_Gatherv(const void *sb, int sc, MPI_Datatype st, void *rb, const int *rc, const int *d,
                MPI_Datatype rt, int root, MPI_Comm c)
{ (void)sb; (void)sc; (void)st; (void)rb; (void)rc; (void)d; (void)rt; (void)root; (void)c; return 0; }
int MPI_Scatterv(const void *sb, const int *sc, const int *d, MPI_Datatype st, void *rb, int rc,
                 MPI_Datatype rt, int root, MPI_Comm c)
{ (void)sb; (void)sc; (void)d; (void)st; (void)rb; (void)rc; (void)rt; (void)root; (void)c; return 0; }

/* render rank (renderer.c:49) */
int start_renderer(void) { return 0; }

/* domain decomposition (geometry.c:29-160): single domain, never called */
void partitionProblem(AABB_t *bg, AABB_t *fg, int *xs, int *lx, float sp, param *p)
{ (void)bg; (void)fg; (void)sp; (void)p; *xs = 0; *lx = 0; }
void setParticleNumbers(AABB_t *bg, AABB_t *fg, edge_t *e, oob_t *o, int nx, float sp, param *p)
{ (void)bg; (void)fg; (void)e; (void)o; (void)nx; (void)sp; (void)p; }
void constructFluidVolume(fluid_particle **pp, fluid_particle *fp, AABB_t *f, int sx, int nx,
                          edge_t *e, float sp, param *p)
{ (void)pp; (void)fp; (void)f; (void)sx; (void)nx; (void)e; (void)sp; (void)p; }

/* halo / migration exchange (communication.c): a single domain has no neighbours */
void createMpiTypes(void) {}
void create_communicators(void) {}
void freeMpiTypes(void) {}
void startHaloExchange(fluid_particle **pp, fluid_particle *fp, edge_t *e, param *p)
{ (void)pp; (void)fp; (void)e; (void)p; }
void finishHaloExchange(fluid_particle **pp, fluid_particle *fp, edge_t *e, param *p)
{ (void)pp; (void)fp; (void)e; (void)p; }
void transferOOBParticles(fluid_particle **pp, fluid_particle *fp, oob_t *o, param *p)
{ (void)pp; (void)fp; (void)o; (void)p; }
