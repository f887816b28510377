# Builds the UNMODIFIED reference RabbitCT sources, where they lie, into
# oracle/_ref/ (git-ignored).  Test infrastructure only: the outputs are used
# to pin the oracle restatement and to make golden fixtures; nothing in the
# product links them.
#
#   make -f oracle/ref.mk            (from the repository root)
#
# Products:
#   oracle/_ref/libref.so      LolaBunny / LolaOMP / LolaOPT / LolaASM +
#                              analyseGeometry (computeLineRanges, shadow)
#   oracle/_ref/rabbitRunner   the reference driver (src/rabbitRunner.c) with
#                              its own registry, for end-to-end runs on .rct files
#   oracle/_ref/rabbitRunnerLolaCUDA
#                              the same driver and modules with the registry of
#                              oracle/registry_lolacuda.c (the reference's table
#                              plus a LolaCUDA row), linked to liblolacuda.so:
#                              the drop-in as a maintainer would build it
#                              (target `lolacuda`, needs the built library)
#
# The reference is plain C + one hand-written SIMD kernel; it is compiled with
# its own flags (mk/include_GCC.mk: -O3 -ffast-math -march=native -std=c99,
# OpenMP on) by gcc directly on its files.  SIMD follows the host: AVX2 on
# x86_64 (mk/config-default.mk VECTORSIZE=8), NEON on aarch64 (VECTORSIZE=4).

REF     ?= /root/reference
SRC     := $(REF)/src
OUT     := oracle/_ref
ARCH    := $(shell uname -m)

ifeq ($(ARCH),x86_64)
SIMD    ?= AVX
else
SIMD    ?= NEON
endif
ifeq ($(SIMD),AVX)
VECSIZE := 8
endif
ifeq ($(SIMD),AVX512)
VECSIZE := 16
endif
ifeq ($(SIMD),SSE)
VECSIZE := 4
endif
ifeq ($(SIMD),NEON)
VECSIZE := 4
endif

CC      := gcc
CFLAGS  := -O3 -ffast-math -march=native -std=c99 -fopenmp -fPIC -D_GNU_SOURCE \
           -DARRAY_ALIGNMENT=64 -DSIMD_NAME=\"$(SIMD)\" -DMAX_NUM_THREADS=32 \
           -DVECTORSIZE=$(VECSIZE) -I$(SRC)

LIB_SRC := LolaBunny.c LolaOMP.c LolaOPT.c LolaASM.c analyseGeometry.c
RUN_SRC := $(filter-out LolaISPC.c,$(notdir $(wildcard $(SRC)/*.c)))
KERNEL  := fastRabbit$(SIMD).S

all: $(OUT)/libref.so $(OUT)/rabbitRunner

$(OUT):
	mkdir -p $(OUT)

$(OUT)/libref.so: $(addprefix $(SRC)/,$(LIB_SRC)) $(SRC)/$(KERNEL) | $(OUT)
	$(CC) $(CFLAGS) -shared -o $@ $(addprefix $(SRC)/,$(LIB_SRC)) $(SRC)/$(KERNEL) -lm

$(OUT)/rabbitRunner: $(addprefix $(SRC)/,$(RUN_SRC)) $(SRC)/$(KERNEL) | $(OUT)
	$(CC) $(CFLAGS) -o $@ $(addprefix $(SRC)/,$(RUN_SRC)) $(SRC)/$(KERNEL) -lm

LOLALIB ?= rabbitct_gb300/_lib
REG_SRC := $(filter-out algorithmRegistry.c,$(RUN_SRC))

lolacuda: $(OUT)/rabbitRunnerLolaCUDA

$(OUT)/rabbitRunnerLolaCUDA: $(addprefix $(SRC)/,$(REG_SRC)) $(SRC)/$(KERNEL) \
		oracle/registry_lolacuda.c $(LOLALIB)/liblolacuda.so | $(OUT)
	$(CC) $(CFLAGS) -o $@ $(addprefix $(SRC)/,$(REG_SRC)) $(SRC)/$(KERNEL) \
		oracle/registry_lolacuda.c -L$(LOLALIB) -llolacuda \
		-Wl,-rpath,$(abspath $(LOLALIB)) -lm -lstdc++ -ldl -lpthread -lrt

clean:
	rm -rf $(OUT)

.PHONY: all clean lolacuda
