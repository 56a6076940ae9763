// Emitted by Reffine's compile path (LoopGen, CanonPass, ReadWritePass, ScalarPass,
// CEmitter) for query `join_agg` of oracle/ref/ref_queries.h, vectorize off; temporaries
// named after heap addresses renumbered.  Regenerate with oracle/ref/emit_generated.py.
// entry: join_agg
#include <algorithm>
#include <cmath>
#include "reffine/vinstr/vinstr.h"

typedef struct {double _0; int64_t _1; } _0_t;

typedef struct {_0_t _0; _0_t _1; _0_t _2; _0_t _3; _0_t _4; } _1_t;

extern "C" void join_agg(_1_t* output_addr, ArrowTable* build, ArrowTable* probe) {
    int64_t _n0[int64_t(1)];
    int64_t* red_idx_addr_n1 = _n0;
    (red_idx_addr_n1)[int64_t(0)] = int64_t(0);
    red_idx_addr_n1;
    ;
    _1_t _n2[int64_t(1)];
    _1_t* state_addr_n3 = _n2;
    ((&(&state_addr_n3->_0)->_0))[int64_t(0)] = double(0.000000);
    (&(&state_addr_n3->_0)->_0);
    ((&(&state_addr_n3->_0)->_1))[int64_t(0)] = int64_t(0);
    (&(&state_addr_n3->_0)->_1);
    ;
    ((&(&state_addr_n3->_1)->_0))[int64_t(0)] = double(0.000000);
    (&(&state_addr_n3->_1)->_0);
    ((&(&state_addr_n3->_1)->_1))[int64_t(0)] = int64_t(0);
    (&(&state_addr_n3->_1)->_1);
    ;
    ((&(&state_addr_n3->_2)->_0))[int64_t(0)] = double(0.000000);
    (&(&state_addr_n3->_2)->_0);
    ((&(&state_addr_n3->_2)->_1))[int64_t(0)] = int64_t(0);
    (&(&state_addr_n3->_2)->_1);
    ;
    ((&(&state_addr_n3->_3)->_0))[int64_t(0)] = double(0.000000);
    (&(&state_addr_n3->_3)->_0);
    ((&(&state_addr_n3->_3)->_1))[int64_t(0)] = int64_t(0);
    (&(&state_addr_n3->_3)->_1);
    ;
    ((&(&state_addr_n3->_4)->_0))[int64_t(0)] = double(0.000000);
    (&(&state_addr_n3->_4)->_0);
    ((&(&state_addr_n3->_4)->_1))[int64_t(0)] = int64_t(0);
    (&(&state_addr_n3->_4)->_1);
    ;
    ;
    
    ;
    #pragma clang loop vectorize(enable) interleave(enable)
    while(1) {
        if (((red_idx_addr_n1)[int64_t(0)] >= get_array_len(get_array_child(get_vector_array(probe), uint32_t(1))))) break;
        
        if (get_null_bit((uint16_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(0)), (red_idx_addr_n1)[int64_t(0)])) {
            ((&(&state_addr_n3->_0)->_0))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(0))) ? (((&(&state_addr_n3->_0)->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) : ((&(&state_addr_n3->_0)->_0))[int64_t(0)]);
            (&(&state_addr_n3->_0)->_0);
            ((&(&state_addr_n3->_0)->_1))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(0))) ? (((&(&state_addr_n3->_0)->_1))[int64_t(0)] + int64_t(1)) : ((&(&state_addr_n3->_0)->_1))[int64_t(0)]);
            (&(&state_addr_n3->_0)->_1);
            ;
            ((&(&state_addr_n3->_1)->_0))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(1))) ? (((&(&state_addr_n3->_1)->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) : ((&(&state_addr_n3->_1)->_0))[int64_t(0)]);
            (&(&state_addr_n3->_1)->_0);
            ((&(&state_addr_n3->_1)->_1))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(1))) ? (((&(&state_addr_n3->_1)->_1))[int64_t(0)] + int64_t(1)) : ((&(&state_addr_n3->_1)->_1))[int64_t(0)]);
            (&(&state_addr_n3->_1)->_1);
            ;
            ((&(&state_addr_n3->_2)->_0))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(2))) ? (((&(&state_addr_n3->_2)->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) : ((&(&state_addr_n3->_2)->_0))[int64_t(0)]);
            (&(&state_addr_n3->_2)->_0);
            ((&(&state_addr_n3->_2)->_1))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(2))) ? (((&(&state_addr_n3->_2)->_1))[int64_t(0)] + int64_t(1)) : ((&(&state_addr_n3->_2)->_1))[int64_t(0)]);
            (&(&state_addr_n3->_2)->_1);
            ;
            ((&(&state_addr_n3->_3)->_0))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(3))) ? (((&(&state_addr_n3->_3)->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) : ((&(&state_addr_n3->_3)->_0))[int64_t(0)]);
            (&(&state_addr_n3->_3)->_0);
            ((&(&state_addr_n3->_3)->_1))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(3))) ? (((&(&state_addr_n3->_3)->_1))[int64_t(0)] + int64_t(1)) : ((&(&state_addr_n3->_3)->_1))[int64_t(0)]);
            (&(&state_addr_n3->_3)->_1);
            ;
            ((&(&state_addr_n3->_4)->_0))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(4))) ? (((&(&state_addr_n3->_4)->_0))[int64_t(0)] + ((double*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(2)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) : ((&(&state_addr_n3->_4)->_0))[int64_t(0)]);
            (&(&state_addr_n3->_4)->_0);
            ((&(&state_addr_n3->_4)->_1))[int64_t(0)] = ((((((vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]]) >= int64_t(0)) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] < int32_t(5))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] >= int32_t(0))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(3)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]] < int32_t(365))) && (((int32_t*) get_array_buf(get_array_child(get_vector_array(build), uint32_t(1)), uint32_t(1)))[vector_locate(build, ((int64_t*) get_array_buf(get_array_child(get_vector_array(probe), uint32_t(1)), uint32_t(1)))[(red_idx_addr_n1)[int64_t(0)]])] == int32_t(4))) ? (((&(&state_addr_n3->_4)->_1))[int64_t(0)] + int64_t(1)) : ((&(&state_addr_n3->_4)->_1))[int64_t(0)]);
            (&(&state_addr_n3->_4)->_1);
            ;
            ;
        } else {
        }
        ;
        (red_idx_addr_n1)[int64_t(0)] = ((red_idx_addr_n1)[int64_t(0)] + int64_t(1));
        red_idx_addr_n1;
        ;
        
    }
    
    _1_t* _red_loop_n4 = state_addr_n3;
    double red_0_0 = ((&(&_red_loop_n4->_0)->_0))[int64_t(0)];
    ((&(&output_addr->_0)->_0))[int64_t(0)] = red_0_0;
    (&(&output_addr->_0)->_0);
    int64_t red_0_1 = ((&(&_red_loop_n4->_0)->_1))[int64_t(0)];
    ((&(&output_addr->_0)->_1))[int64_t(0)] = red_0_1;
    (&(&output_addr->_0)->_1);
    ;
    double red_1_0 = ((&(&_red_loop_n4->_1)->_0))[int64_t(0)];
    ((&(&output_addr->_1)->_0))[int64_t(0)] = red_1_0;
    (&(&output_addr->_1)->_0);
    int64_t red_1_1 = ((&(&_red_loop_n4->_1)->_1))[int64_t(0)];
    ((&(&output_addr->_1)->_1))[int64_t(0)] = red_1_1;
    (&(&output_addr->_1)->_1);
    ;
    double red_2_0 = ((&(&_red_loop_n4->_2)->_0))[int64_t(0)];
    ((&(&output_addr->_2)->_0))[int64_t(0)] = red_2_0;
    (&(&output_addr->_2)->_0);
    int64_t red_2_1 = ((&(&_red_loop_n4->_2)->_1))[int64_t(0)];
    ((&(&output_addr->_2)->_1))[int64_t(0)] = red_2_1;
    (&(&output_addr->_2)->_1);
    ;
    double red_3_0 = ((&(&_red_loop_n4->_3)->_0))[int64_t(0)];
    ((&(&output_addr->_3)->_0))[int64_t(0)] = red_3_0;
    (&(&output_addr->_3)->_0);
    int64_t red_3_1 = ((&(&_red_loop_n4->_3)->_1))[int64_t(0)];
    ((&(&output_addr->_3)->_1))[int64_t(0)] = red_3_1;
    (&(&output_addr->_3)->_1);
    ;
    double red_4_0 = ((&(&_red_loop_n4->_4)->_0))[int64_t(0)];
    ((&(&output_addr->_4)->_0))[int64_t(0)] = red_4_0;
    (&(&output_addr->_4)->_0);
    int64_t red_4_1 = ((&(&_red_loop_n4->_4)->_1))[int64_t(0)];
    ((&(&output_addr->_4)->_1))[int64_t(0)] = red_4_1;
    (&(&output_addr->_4)->_1);
    ;
    ;
    ;
}