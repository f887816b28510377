/* The reference runner's algorithm table with LolaCUDA as one more row: what a
 * maintainer's change to src/algorithmRegistry.c amounts to, written as a unit
 * of its own so that the reference runner can be linked against
 * liblolacuda.so without touching the reference sources (oracle/ref.mk,
 * target rabbitRunnerLolaCUDA).  Test infrastructure: it proves the drop-in at
 * link and call level; the product does not use it.
 *
 * Interface kept alike, because the runner binds to it by name
 * (src/algorithmRegistry.h:18-23, used at src/rabbitRunner.c:183-232): the
 * three global entry-point pointers and algorithmRegistryFind / List. */
#include <stdio.h>
#include <string.h>

#include "algorithmRegistry.h"

int lolaOmpPrepare(RabbitCtGlobalData *);
int lolaOmpBackprojection(RabbitCtGlobalData *);
int lolaOmpFinish(RabbitCtGlobalData *);
int lolaBunnyPrepare(RabbitCtGlobalData *);
int lolaBunnyBackprojection(RabbitCtGlobalData *);
int lolaBunnyFinish(RabbitCtGlobalData *);
int lolaOptPrepare(RabbitCtGlobalData *);
int lolaOptBackprojection(RabbitCtGlobalData *);
int lolaOptFinish(RabbitCtGlobalData *);
int lolaAsmPrepare(RabbitCtGlobalData *);
int lolaAsmBackprojection(RabbitCtGlobalData *);
int lolaAsmFinish(RabbitCtGlobalData *);
/* include/lolaCuda.h declares the same three (the headers share the
   RabbitCtGlobalData guard); declared here to keep this unit self-contained */
int lolaCudaPrepare(RabbitCtGlobalData *);
int lolaCudaBackprojection(RabbitCtGlobalData *);
int lolaCudaFinish(RabbitCtGlobalData *);

FncPrepareAlgorithmType FncPrepareAlgorithm;
FncAlgorithmIterationType FncAlgorithmIteration;
FncFinishAlgorithmType FncFinishAlgorithm;

static const AlgorithmEntryType kModules[] = {
  { "LolaOMP", lolaOmpPrepare, lolaOmpBackprojection, lolaOmpFinish },
  { "LolaBunny", lolaBunnyPrepare, lolaBunnyBackprojection, lolaBunnyFinish },
  { "LolaOPT", lolaOptPrepare, lolaOptBackprojection, lolaOptFinish },
  { "LolaASM", lolaAsmPrepare, lolaAsmBackprojection, lolaAsmFinish },
  { "LolaCUDA", lolaCudaPrepare, lolaCudaBackprojection, lolaCudaFinish },
};

void algorithmRegistryList(void)
{
  printf("Available algorithms:\n");
  for (size_t i = 0; i < sizeof(kModules) / sizeof(kModules[0]); ++i)
    printf("  %s\n", kModules[i].name);
}

int algorithmRegistryFind(const char *name)
{
  for (size_t i = 0; i < sizeof(kModules) / sizeof(kModules[0]); ++i) {
    if (strcmp(kModules[i].name, name) != 0)
      continue;
    FncPrepareAlgorithm = kModules[i].prepare;
    FncAlgorithmIteration = kModules[i].iterate;
    FncFinishAlgorithm = kModules[i].finish;
    return 1;
  }
  printf("Unknown algorithm: %s\n", name);
  algorithmRegistryList();
  return 0;
}
