# Compiles the reference primecount (CPU, OpenMP) from its own sources into
# oracle/_ref/.  This is test infrastructure: the binary is the checker used to
# generate golden fixtures, to validate the C restatement in
# oracle/pcg_oracle.c, and the timed CPU reference of bench.py.  Nothing in
# the product links it.
#
#   make -f oracle/ref.mk REF=<primecount source tree> -j8       # build
#   make -f oracle/ref.mk REF=<primecount source tree> stage      # see below
#
# REF defaults to $(PCG_REFERENCE).  The flags follow the reference's CMake
# Release build: -O3, OpenMP, libdivide, int128, and its run-time CPU
# dispatch (ENABLE_MULTIARCH_*) where the compiler supports the target
# attribute -- AVX512 VPOPCNTDQ on x86-64, SVE on aarch64 (the reference's
# cmake/multiarch_*.cmake decide the same way; SVE also needs a host CPU
# that reports it, see below).
#
# `stage` copies the source files this recipe compiles into $(STAGE) (a
# git-ignored directory, never committed), so that a host without the
# reference tree (the aarch64 GPU host) can build the reference with
# REF=$(STAGE).
#
# Output: $(OUT)/primecount (CLI) and $(OUT)/libprimecount_ref.a, one
# directory per CPU architecture.
REF    ?= $(PCG_REFERENCE)
ARCH   := $(shell uname -m)
OUT    ?= oracle/_ref/$(ARCH)
STAGE  ?= oracle/_ref/src
CXX    ?= g++
HERE   := $(dir $(lastword $(MAKEFILE_LIST)))

ifeq ($(strip $(REF)),)
$(error set REF=<primecount source tree> or PCG_REFERENCE)
endif

CXXFLAGS ?= -O3 -std=gnu++17 -fopenmp -DNDEBUG
DEFS   := -DENABLE_LIBDIVIDE
PS_DEFS :=
ARCH_SRC :=
PS_ARCH_SRC :=

# run-time dispatch: only when the compiler accepts the probe
ifeq ($(ARCH),x86_64)
ifeq ($(shell $(CXX) -std=gnu++17 -c -x c++ $(HERE)probe_avx512.cpp -o /dev/null 2>/dev/null && echo 1),1)
DEFS    += -DENABLE_MULTIARCH_x86_POPCNT -DENABLE_MULTIARCH_AVX512_VPOPCNT
PS_DEFS += -DENABLE_MULTIARCH_x86_POPCNT -DENABLE_MULTIARCH_AVX512_BW -DENABLE_MULTIARCH_AVX512_VBMI2
ARCH_SRC := $(REF)/src/arch/x86/cpuid.cpp
PS_ARCH_SRC := $(REF)/lib/primesieve/src/arch/x86/cpuid.cpp
endif
endif
# aarch64: SVE dispatch only where the host's CPU reports SVE (the Grace cores
# of the GB300 host do not expose it, and a build with SVE dispatch compiled
# in died there with SIGILL; without it the reference runs its default path)
SVE_HOST := $(shell grep -qw sve /proc/cpuinfo 2>/dev/null && echo 1)
ifeq ($(ARCH)$(SVE_HOST),aarch641)
ifeq ($(shell $(CXX) -std=gnu++17 -c -x c++ $(HERE)probe_sve.cpp -o /dev/null 2>/dev/null && echo 1),1)
DEFS    += -DENABLE_MULTIARCH_ARM_SVE
PS_DEFS += -DENABLE_MULTIARCH_ARM_SVE
ARCH_SRC := $(REF)/src/arch/arm/sve.cpp
PS_ARCH_SRC := $(REF)/lib/primesieve/src/arch/arm/sve.cpp
endif
endif

INC    := -I$(REF)/include -I$(REF)/src -I$(REF)/lib/primesieve/include -I$(REF)/lib/primesieve/src

PC_SRC := $(filter-out $(REF)/src/app/%,$(wildcard $(REF)/src/*.cpp) \
          $(REF)/src/sieve/Sieve.cpp $(REF)/src/sieve/pre_sieve.cpp \
          $(wildcard $(REF)/src/lmo/*.cpp) $(wildcard $(REF)/src/deleglise-rivat/*.cpp) \
          $(wildcard $(REF)/src/gourdon/*.cpp)) $(ARCH_SRC)
PS_SRC := $(wildcard $(REF)/lib/primesieve/src/*.cpp) $(PS_ARCH_SRC)
APP_SRC := $(wildcard $(REF)/src/app/*.cpp)

PC_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(PC_SRC))
PS_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(PS_SRC))
APP_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(APP_SRC))

all: $(OUT)/primecount $(OUT)/libprimecount_ref.a $(OUT)/build_flags.txt

$(OUT)/obj/lib/primesieve/%.o: $(REF)/lib/primesieve/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(PS_DEFS) $(INC) -c $< -o $@

$(OUT)/obj/src/%.o: $(REF)/src/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -c $< -o $@

$(OUT)/libprimecount_ref.a: $(PC_OBJ) $(PS_OBJ)
	ar rcs $@ $^

$(OUT)/primecount: $(APP_OBJ) $(OUT)/libprimecount_ref.a
	$(CXX) $(CXXFLAGS) $(APP_OBJ) $(OUT)/libprimecount_ref.a -o $@

$(OUT)/build_flags.txt: $(OUT)/primecount
	@echo "arch=$(ARCH) cxx=$$($(CXX) -dumpfullversion) flags=$(CXXFLAGS) defs=$(DEFS) primesieve_defs=$(PS_DEFS)" > $@

# Integration check: the reference's own test programs for the hard leaves
# (test/gourdon/D.cpp, test/deleglise-rivat/S2_hard_alpha.cpp,
# test/gourdon/pi_gourdon.cpp), linked with the drop-in D() / S2_hard() of
# primecount_gb300/integration/hard_leaves_gpu.cpp (which calls libpcgpu)
# and with the reference's own bodies renamed D_cpu / S2_hard_cpu.
#   make -f oracle/ref.mk REF=... itest PCGPU=<repository root>
PCGPU  ?= .
ITEST  := $(OUT)/itest
ITEST_PROGS := $(ITEST)/test_D $(ITEST)/test_S2_hard_alpha $(ITEST)/test_pi_gourdon
NOHARD_OBJ := $(filter-out %/gourdon/D.o %/deleglise-rivat/S2_hard.o,$(PC_OBJ)) $(PS_OBJ)

itest: $(ITEST_PROGS)

$(ITEST)/D_cpu.o: $(REF)/src/gourdon/D.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -DD=D_cpu -c $< -o $@

$(ITEST)/S2_hard_cpu.o: $(REF)/src/deleglise-rivat/S2_hard.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -DS2_hard=S2_hard_cpu -c $< -o $@

$(ITEST)/hard_leaves_gpu.o: $(PCGPU)/primecount_gb300/integration/hard_leaves_gpu.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) -I$(PCGPU)/include -c $< -o $@

$(ITEST)/libref_nohard.a: $(NOHARD_OBJ)
	@mkdir -p $(dir $@)
	rm -f $@ && ar rcs $@ $^

ITEST_LINK := $(ITEST)/hard_leaves_gpu.o $(ITEST)/D_cpu.o $(ITEST)/S2_hard_cpu.o $(ITEST)/libref_nohard.a \
              -L$(abspath $(PCGPU))/primecount_gb300 -lpcgpu -Wl,-rpath,$(abspath $(PCGPU))/primecount_gb300

$(ITEST)/test_D: $(REF)/test/gourdon/D.cpp $(ITEST)/hard_leaves_gpu.o $(ITEST)/D_cpu.o $(ITEST)/S2_hard_cpu.o $(ITEST)/libref_nohard.a
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) $< $(ITEST_LINK) -o $@

$(ITEST)/test_S2_hard_alpha: $(REF)/test/deleglise-rivat/S2_hard_alpha.cpp $(ITEST)/hard_leaves_gpu.o $(ITEST)/D_cpu.o $(ITEST)/S2_hard_cpu.o $(ITEST)/libref_nohard.a
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) $< $(ITEST_LINK) -o $@

$(ITEST)/test_pi_gourdon: $(REF)/test/gourdon/pi_gourdon.cpp $(ITEST)/hard_leaves_gpu.o $(ITEST)/D_cpu.o $(ITEST)/S2_hard_cpu.o $(ITEST)/libref_nohard.a
	$(CXX) $(CXXFLAGS) $(DEFS) $(INC) $< $(ITEST_LINK) -o $@

# the sources compiled above plus the headers they include
stage:
	@mkdir -p $(STAGE)
	cd $(REF) && cp -r --parents include src lib/primesieve/include lib/primesieve/src \
	  test/gourdon/D.cpp test/deleglise-rivat/S2_hard_alpha.cpp test/gourdon/pi_gourdon.cpp COPYING $(abspath $(STAGE))/

.PHONY: all stage itest
