/* vsg/vsgpackedmsg.h -- TEST INFRASTRUCTURE: MPI messages are not used (no VSG_HAVE_MPI). */
