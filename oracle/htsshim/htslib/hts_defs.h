/* Oracle test infrastructure: project-written stand-in for the htslib
 * header of the same name.  htslib is not installed in this environment;
 * this shim provides only the subset of the public htslib API that the
 * RabbitVar sources call, re-implemented from the SAM/BAM/BGZF/FAI
 * specifications.  It is used only to build the reference as an oracle. */
#ifndef RV_SHIM_HTS_DEFS_H
#define RV_SHIM_HTS_DEFS_H
#endif
