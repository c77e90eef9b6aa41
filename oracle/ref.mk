# Compiles the reference primecount (CPU, OpenMP) from its own sources, where
# they lie, into oracle/_ref/.  This is test infrastructure: the binary is the
# checker used to generate golden fixtures and to validate the C restatement in
# oracle/pcg_oracle.c.  Nothing in the product links it.
#
#   make -f oracle/ref.mk REF=/root/reference -j8
#
# Output: oracle/_ref/primecount (CLI) and oracle/_ref/libprimecount_ref.a
REF    ?= /root/reference
OUT    ?= oracle/_ref
CXX    ?= g++
CXXFLAGS ?= -O2 -std=gnu++17 -fopenmp -DNDEBUG
INC    := -I$(REF)/include -I$(REF)/src -I$(REF)/lib/primesieve/include

PC_SRC := $(filter-out $(REF)/src/app/%,$(wildcard $(REF)/src/*.cpp) \
          $(REF)/src/sieve/Sieve.cpp $(REF)/src/sieve/pre_sieve.cpp \
          $(wildcard $(REF)/src/lmo/*.cpp) $(wildcard $(REF)/src/deleglise-rivat/*.cpp) \
          $(wildcard $(REF)/src/gourdon/*.cpp))
PS_SRC := $(wildcard $(REF)/lib/primesieve/src/*.cpp)
APP_SRC := $(wildcard $(REF)/src/app/*.cpp)

PC_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(PC_SRC))
PS_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(PS_SRC))
APP_OBJ := $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(APP_SRC))

all: $(OUT)/primecount $(OUT)/libprimecount_ref.a

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/libprimecount_ref.a: $(PC_OBJ) $(PS_OBJ)
	ar rcs $@ $^

$(OUT)/primecount: $(APP_OBJ) $(OUT)/libprimecount_ref.a
	$(CXX) $(CXXFLAGS) $(APP_OBJ) $(OUT)/libprimecount_ref.a -o $@

.PHONY: all
