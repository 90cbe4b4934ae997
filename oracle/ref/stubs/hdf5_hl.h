/* Empty stand-in for <hdf5_hl.h> (oracle/_ref harness only). */
