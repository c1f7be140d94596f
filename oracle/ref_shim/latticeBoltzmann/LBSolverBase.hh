/* Empty stand-in: topOpt/checkpointingBase.hh includes this header but uses
 * nothing from it. */
#ifndef LBSOLVERBASE
#define LBSOLVERBASE
#endif
