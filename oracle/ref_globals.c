/* Process-rank globals that the reference defines in its main.c.  The
 * reference checker library (oracle/_ref/libemmi_ref.so) links every
 * reference source except main.c, so it needs them from here: one rank. */
int iproc = 0, nproc = 1, ierr = 0;
