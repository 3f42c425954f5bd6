# Builds the UNMODIFIED reference C core (REBOUND 5.0.0) from its own source
# files, in place where they lie, into oracle/_ref/.  Test infrastructure only:
# the product never links or loads anything built here.
#
#   make -f oracle/ref.mk REF=<reference checkout>
#
# Outputs (git-ignored):
#   oracle/_ref/librebound$(EXT_SUFFIX)   serial, -ffp-contract=off (parity build;
#                                         importable as the `librebound` module the
#                                         reference's Python package looks for)
#   oracle/_ref/librebound_omp.so         OpenMP build (-DOPENMP), for timing
#   oracle/_ref/librebound_quad.so        serial parity build with -DQUADRUPOLE (the
#                                         reference's compile-time quadrupole tree,
#                                         src/Makefile.defs:90-91), for fixtures
#
# The recipe compiles every src/*.c like the reference's setup.py does, without
# the HTTP server (-DSERVER is omitted) and without OpenGL.
ifndef REF
$(error REF=<reference checkout> is required)
endif
OUT := oracle/_ref
EXT_SUFFIX := $(shell python3 -c "import sysconfig;print(sysconfig.get_config_var('EXT_SUFFIX') or '.so')")
SRCS := $(filter-out $(REF)/src/server.c,$(sort $(wildcard $(REF)/src/*.c)))
CFLAGS := -std=c99 -O3 -fPIC -D_GNU_SOURCE -fstrict-aliasing -Wno-unknown-pragmas \
          -Wno-unreachable-code -DGITHASH=reference -I$(REF)/src

all: $(OUT)/librebound$(EXT_SUFFIX) $(OUT)/librebound_omp.so $(OUT)/librebound_quad.so

$(OUT)/librebound$(EXT_SUFFIX): $(SRCS)
	@mkdir -p $(OUT)
	$(CC) $(CFLAGS) -ffp-contract=off -shared $(SRCS) -lm -o $@

$(OUT)/librebound_omp.so: $(SRCS)
	@mkdir -p $(OUT)
	$(CC) $(CFLAGS) -DOPENMP -fopenmp -shared $(SRCS) -lm -fopenmp -o $@

$(OUT)/librebound_quad.so: $(SRCS)
	@mkdir -p $(OUT)
	$(CC) $(CFLAGS) -ffp-contract=off -DQUADRUPOLE -shared $(SRCS) -lm -o $@

.PHONY: all
