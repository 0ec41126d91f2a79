/* vsg/vsgmpi.h -- TEST INFRASTRUCTURE: MPI is not used (no VSG_HAVE_MPI). */
